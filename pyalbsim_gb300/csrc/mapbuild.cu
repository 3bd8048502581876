// Photon-map index build: the GPU replacement of build_photon_map_data + PhotonMapIndex
// (alb_sim/photon_mapping/build_photon_map_data.py:8-62, photon_map_index.py:6-17).
//
// Records are put in an exact left-balanced k-d order (median splits on each node's widest
// axis, 32-record leaves; streaming partition passes over the whole map for the upper levels,
// one CTA per node of at most 4096 records for the rest), permuted into that order as two
// float4 streams, and cut into leaves of 32 consecutive records. A leaf's bounding box is a
// leaf box; 32 consecutive boxes form the next level up, until 32 or fewer boxes remain. The
// gather walks this implicit 32-ary box tree warp-wide. The same file sorts the gather
// queries along a Morton curve (LSD radix sort of interleaved cell coordinates).
#include <atomic>
#include <algorithm>
#include <cstdio>

#include "device_common.cuh"
#include "internal.h"

namespace alb {

// ------------------------------------------------------------------------------------------
// bounding box
// ------------------------------------------------------------------------------------------

ALB_DEVICE unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
ALB_HOST_DEVICE float ord2f(unsigned u) {
    unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

// box[0..2] = ordered-min of x,y,z, box[3..5] = ordered-max; initialised to (~0, 0).
__global__ void k_bbox(const float4* __restrict__ a, uint64_t stride, uint64_t n, unsigned* box) {
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float4 p = a[i * stride];
        float x = p.x, y = p.y, z = p.z;
        lo[0] = fminf(lo[0], x); hi[0] = fmaxf(hi[0], x);
        lo[1] = fminf(lo[1], y); hi[1] = fmaxf(hi[1], y);
        lo[2] = fminf(lo[2], z); hi[2] = fmaxf(hi[2], z);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    // the block's warps meet in shared memory: one set of global atomics per block (they
    // all land on the same six words)
    __shared__ unsigned sb[6];
    if (threadIdx.x < 6) sb[threadIdx.x] = threadIdx.x < 3 ? 0xffffffffu : 0u;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(sb + k, f2ord(lo[k]));
            atomicMax(sb + 3 + k, f2ord(hi[k]));
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) atomicMin(box + threadIdx.x, sb[threadIdx.x]);
    else if (threadIdx.x < 6) atomicMax(box + threadIdx.x, sb[threadIdx.x]);
}

// ------------------------------------------------------------------------------------------
// Morton keys
// ------------------------------------------------------------------------------------------

ALB_DEVICE uint64_t spread2(uint64_t x) {  // 32 bits -> even bits of 64
    x &= 0x00000000ffffffffull;
    x = (x | (x << 16)) & 0x0000ffff0000ffffull;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}
ALB_DEVICE uint64_t spread3(uint64_t x) {  // 21 bits -> every third bit of 63
    x &= 0x1fffffull;
    x = (x | (x << 32)) & 0x001f00000000ffffull;
    x = (x | (x << 16)) & 0x001f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// 64-bit Morton cell key: 21 bits per axis in 3-D, 32 bits per axis for planar maps.
ALB_DEVICE uint64_t morton_key(const KeyGrid& g, float x, float y, float z) {
    float v[3] = {x, y, z};
    uint64_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double t = ((double)v[k] - g.lo[k]) * g.scale[k];
        t = fmin(fmax(t, 0.0), g.maxq[k]);
        q[k] = (uint64_t)t;
    }
    if (g.naxes == 3) return spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
    if (g.naxes == 2) return spread2(q[g.ax[0]]) | (spread2(q[g.ax[1]]) << 1);
    if (g.naxes == 1) return q[g.ax[0]];
    return 0ull;
}

// Query sort keys: 32-bit Morton codes (the query grid has at most 10 bits per axis in 3-D
// and 16 in 2-D).
__global__ void k_keys(const float4* __restrict__ a, uint64_t n, KeyGrid g, uint32_t* keys, uint32_t* vals,
                       unsigned long long* or_and) {
    unsigned long long o = 0ull, an = ~0ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float4 p = a[i];
        const uint32_t key = (uint32_t)morton_key(g, p.x, p.y, p.z);
        keys[i] = key;
        vals[i] = (uint32_t)i;
        o |= key;
        an &= key;
    }
    for (int s = 16; s > 0; s >>= 1) {
        o |= __shfl_xor_sync(0xffffffffu, o, s);
        an &= __shfl_xor_sync(0xffffffffu, an, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicOr(or_and, o);
        atomicAnd(or_and + 1, an);
    }
}

// ------------------------------------------------------------------------------------------
// LSD radix sort of (u32 key, u32 value), 8-bit digits, stable.
// Tile = 8 warps x 16 rounds x 32 lanes; key t of warp w, round j, lane l is
// tile_base + w*512 + j*32 + l, so ranking warps in order, rounds in order and lanes in
// order preserves the input order of equal digits.
// ------------------------------------------------------------------------------------------
constexpr int kRsWarps = 8, kRsItems = 16, kRsThreads = kRsWarps * 32;
constexpr int kRsTile = kRsThreads * kRsItems;

template <class K>
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const K* __restrict__ keys, uint64_t n,
                                                         int shift, uint32_t* hist, uint32_t ntiles) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * kRsTile;
    for (int j = threadIdx.x; j < kRsTile; j += kRsThreads) {
        uint64_t i = base + j;
        if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kRsThreads) hist[(uint64_t)d * ntiles + blockIdx.x] = h[d];
}

template <class K>
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const K* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            K* __restrict__ kout,
                                                            uint32_t* __restrict__ vout, uint64_t n,
                                                            int shift, const uint32_t* __restrict__ offs,
                                                            uint32_t ntiles) {
    __shared__ uint32_t wcnt[kRsWarps][256];
    __shared__ uint32_t goff[256];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wcnt[0][0])[i] = 0;
    for (int d = threadIdx.x; d < 256; d += kRsThreads) goff[d] = offs[(uint64_t)d * ntiles + blockIdx.x];
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kRsTile + (uint64_t)w * (kRsItems * 32);
    K key[kRsItems];
    uint32_t val[kRsItems], rank[kRsItems];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        uint64_t i = base + (uint64_t)j * 32 + l;
        bool valid = i < n;
        key[j] = valid ? kin[i] : (K)0;
        val[j] = valid ? vin[i] : 0u;
        unsigned act = __ballot_sync(0xffffffffu, valid);
        rank[j] = 0;
        if (valid) {
            uint32_t d = (uint32_t)(key[j] >> shift) & 255u;
            unsigned peers = __match_any_sync(act, d);
            uint32_t cur = wcnt[w][d];
            __syncwarp(act);
            rank[j] = cur + __popc(peers & lt);
            if (l == __ffs(peers) - 1) wcnt[w][d] = cur + __popc(peers);
            __syncwarp(act);
        }
    }
    __syncthreads();
    if (threadIdx.x < 256) {
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kRsWarps; ++ww) {
            uint32_t c = wcnt[ww][threadIdx.x];
            wcnt[ww][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        uint64_t i = base + (uint64_t)j * 32 + l;
        if (i < n) {
            uint32_t d = (uint32_t)(key[j] >> shift) & 255u;
            uint32_t dst = goff[d] + wcnt[w][d] + rank[j];
            kout[dst] = key[j];
            vout[dst] = val[j];
        }
    }
}

// Exclusive scan of u32 (device-wide, recursive over block sums).
constexpr int kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_tile(uint32_t* data, uint64_t n, uint32_t* sums) {
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t acc = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        uint64_t i = base + j;
        v[j] = i < n ? data[i] : 0u;
        acc += v[j];
    }
    // exclusive scan of per-thread totals across the block
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = acc;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (l >= o) incl += t;
    }
    if (l == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t t = l < kScanThreads / 32 ? warp_tot[l] : 0u;
        uint32_t ti = t;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, ti, o);
            if (l >= o) ti += u;
        }
        if (l < kScanThreads / 32) warp_tot[l] = ti - t;
        if (l == kScanThreads / 32 - 1 && sums) sums[blockIdx.x] = ti;
    }
    __syncthreads();
    uint32_t run = warp_tot[w] + incl - acc;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        uint64_t i = base + j;
        if (i < n) data[i] = run;
        run += v[j];
    }
}

__global__ void k_scan_add(uint32_t* data, uint64_t n, const uint32_t* sums) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) data[i] += sums[i / kScanTile];
}

// Returns -1 when a temporary could not be allocated (nothing is launched on it).
static int exclusive_scan(Workspace& ws, uint32_t* data, uint64_t n, cudaStream_t st) {
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles <= 1) {
        k_scan_tile<<<1, kScanThreads, 0, st>>>(data, n, nullptr);
        note_launch();
        return 0;
    }
    uint32_t* sums = ws.take_u32(tiles);
    if (!sums) return -1;
    k_scan_tile<<<(unsigned)tiles, kScanThreads, 0, st>>>(data, n, sums);
    note_launch();
    if (exclusive_scan(ws, sums, tiles, st) != 0) return -1;
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(data, n, sums);
    note_launch();
    return 0;
}

template <class K>
static int radix_sort_pairs(Workspace& ws, K*& keys, uint32_t*& vals, K*& keys_alt, uint32_t*& vals_alt, uint64_t n,
                            uint64_t varying_bits, cudaStream_t st) {
    if (n <= 1) return 0;
    const uint32_t ntiles = (uint32_t)((n + kRsTile - 1) / kRsTile);
    size_t mark = ws.mark();
    uint32_t* hist = ws.take_u32((uint64_t)ntiles * 256);
    if (!hist) {
        ws.release(mark);
        return -1;
    }
    int passes = 0;
    for (int shift = 0; shift < (int)(8 * sizeof(K)); shift += 8) {
        if (((varying_bits >> shift) & 255ull) == 0ull) continue;  // digit constant over all keys
        k_rs_hist<<<ntiles, kRsThreads, 0, st>>>(keys, n, shift, hist, ntiles);
        note_launch();
        if (exclusive_scan(ws, hist, (uint64_t)ntiles * 256, st) != 0) {
            ws.release(mark);
            return -1;
        }
        k_rs_scatter<<<ntiles, kRsThreads, 0, st>>>(keys, vals, keys_alt, vals_alt, n, shift, hist, ntiles);
        note_launch();
        std::swap(keys, keys_alt);
        std::swap(vals, vals_alt);
        ++passes;
    }
    ws.release(mark);
    return passes;
}

// ------------------------------------------------------------------------------------------
// k-d order: a left-balanced median-split k-d tree over 32-record leaves. A node holding
// c leaves gives its left child the largest power of two below c, so every aligned run of
// 32^j leaves is one k-d subtree and the implicit 32-ary box tree inherits k-d cells
// (tight, non-overlapping boxes) instead of Morton runs that straddle far-apart cells.
// Every split cuts the node's widest box axis at the 16-bit quantised coordinate that
// leaves exactly the left child's record count on its side.
// ------------------------------------------------------------------------------------------

ALB_DEVICE void kd_node(uint64_t leaf, uint64_t L, int depth, uint64_t& a, uint64_t& c) {
    a = 0;
    c = L;
    for (int i = 0; i < depth && c > 1; ++i) {
        uint64_t left = 1ull << (63 - __clzll((long long)(c - 1)));
        if (leaf - a < left) {
            c = left;
        } else {
            a += left;
            c -= left;
        }
    }
}

constexpr int kCellMax = 4096;  // records of one node ordered by one CTA in shared memory
constexpr int kCellThreads = 512;
constexpr uint32_t kDummy = 0xffffffffu;

static size_t cell_smem_bytes() {
    return (size_t)kCellMax * 8 + (size_t)kCellMax * 16 + (size_t)2 * 3 * (kCellMax / 32) * 4;
}

struct CellSmem {
    unsigned long long* key;  // kCellMax sort keys
    float *X, *Y, *Z;         // kCellMax coordinates
    uint32_t* ID;             // kCellMax record ids
    unsigned *blo, *bhi;      // 3 * (kCellMax / 32) ordered-int node boxes
};

ALB_DEVICE CellSmem cell_smem(unsigned char* raw) {
    CellSmem s;
    s.key = (unsigned long long*)raw;
    s.X = (float*)(s.key + kCellMax);
    s.Y = s.X + kCellMax;
    s.Z = s.Y + kCellMax;
    s.ID = (uint32_t*)(s.Z + kCellMax);
    s.blo = (unsigned*)(s.ID + kCellMax);
    s.bhi = s.blo + 3 * (kCellMax / 32);
    return s;
}

// Exact left-balanced k-d order of one node's records held in shared memory: entries
// [0, cnt) are records, [cnt, P) (P = cnt rounded up to 32) dummies with NaN positions.
// Reorders X/Y/Z/ID in place, level by level: node boxes -> key (node, 16-bit coordinate
// on the node's widest axis, slot) -> bitonic sort -> permute. Dummies sort last inside
// their node, so they stay in the last leaf. Called by every thread of the CTA.
ALB_DEVICE void cell_kd_sort(const CellSmem& s, unsigned cnt) {
    const unsigned P = (cnt + 31u) & ~31u;
    const unsigned Lc = P / 32;
    unsigned P2 = 32;
    while (P2 < P) P2 <<= 1;
    int depth = 0;
    while ((1u << depth) < Lc) ++depth;
    // In a full cell of a power-of-two leaf count every node of level d is an aligned block
    // of P >> d keys: sorting the blocks separately gives the same order as the full sort.
    const bool perfect = cnt == P && (Lc & (Lc - 1)) == 0;
    for (int d = 0; d < depth; ++d) {
        const unsigned S = perfect ? (P >> d) : P2;
        for (unsigned i = threadIdx.x; i < 3 * Lc; i += blockDim.x) {
            s.blo[i] = 0xffffffffu;
            s.bhi[i] = 0u;
        }
        __syncthreads();
        for (unsigned j = threadIdx.x; j < cnt; j += blockDim.x) {
            uint64_t na, nc;
            kd_node(j / 32, Lc, d, na, nc);
            if (nc > 1) {
                atomicMin(s.blo + 3 * na, f2ord(s.X[j])); atomicMax(s.bhi + 3 * na, f2ord(s.X[j]));
                atomicMin(s.blo + 3 * na + 1, f2ord(s.Y[j])); atomicMax(s.bhi + 3 * na + 1, f2ord(s.Y[j]));
                atomicMin(s.blo + 3 * na + 2, f2ord(s.Z[j])); atomicMax(s.bhi + 3 * na + 2, f2ord(s.Z[j]));
            }
        }
        __syncthreads();
        for (unsigned j = threadIdx.x; j < P2; j += blockDim.x) {
            unsigned long long k = ~0ull;
            if (j < P) {
                uint64_t na, nc;
                kd_node(j / 32, Lc, d, na, nc);
                uint64_t q = 0;
                if (j >= cnt) {
                    q = 0x1ffff;
                } else if (nc > 1) {
                    const unsigned* lo = s.blo + 3 * na;
                    const unsigned* hi = s.bhi + 3 * na;
                    float l0 = ord2f(lo[0]), l1 = ord2f(lo[1]), l2 = ord2f(lo[2]);
                    float e0 = ord2f(hi[0]) - l0, e1 = ord2f(hi[1]) - l1, e2 = ord2f(hi[2]) - l2;
                    float v, l, e;
                    if (e0 >= e1 && e0 >= e2) { v = s.X[j]; l = l0; e = e0; }
                    else if (e1 >= e2) { v = s.Y[j]; l = l1; e = e1; }
                    else { v = s.Z[j]; l = l2; e = e2; }
                    if (e > 0.f) q = (uint64_t)fminf(fmaxf((v - l) / e * 65535.f, 0.f), 65535.f);
                }
                k = (((na << 17) | q) << 13) | j;  // j < 8192 keeps equal keys in place
            }
            s.key[j] = k;
        }
        __syncthreads();
        // bitonic sort of every aligned block of S keys, ascending (the last merge of a block
        // runs ascending everywhere)
        for (unsigned kk = 2; kk <= S; kk <<= 1) {
            for (unsigned jj = kk >> 1; jj > 0; jj >>= 1) {
                for (unsigned i = threadIdx.x; i < P2; i += blockDim.x) {
                    unsigned p = i ^ jj;
                    if (p > i) {
                        unsigned long long x = s.key[i], y = s.key[p];
                        bool up = kk == S || (i & kk) == 0;
                        if ((x > y) == up) {
                            s.key[i] = y;
                            s.key[p] = x;
                        }
                    }
                }
                __syncthreads();
            }
        }
        constexpr int R = kCellMax / kCellThreads;  // each thread stages its slots in registers
        float rx[R], ry[R], rz[R];
        uint32_t rid[R];
#pragma unroll
        for (int t = 0; t < R; ++t) {
            unsigned j = threadIdx.x + t * kCellThreads;
            if (j < P) {
                unsigned src = (unsigned)(s.key[j] & 0x1fffull);
                rx[t] = s.X[src]; ry[t] = s.Y[src]; rz[t] = s.Z[src]; rid[t] = s.ID[src];
            }
        }
        __syncthreads();
#pragma unroll
        for (int t = 0; t < R; ++t) {
            unsigned j = threadIdx.x + t * kCellThreads;
            if (j < P) {
                s.X[j] = rx[t]; s.Y[j] = ry[t]; s.Z[j] = rz[t]; s.ID[j] = rid[t];
            }
        }
        __syncthreads();
    }
}

// One cell of records a[perm[start + j]], j < count (<= kCellMax): writes its padded k-d
// order (kDummy for padding) to out[pstart ..]. Used by the allocation-free k-NN index.
__global__ void __launch_bounds__(kCellThreads) k_cell_kd(const float4* __restrict__ a, const uint32_t* __restrict__ perm,
                                                          const unsigned* __restrict__ start,
                                                          const unsigned* __restrict__ count,
                                                          const unsigned* __restrict__ pstart, uint32_t* out) {
    extern __shared__ unsigned char smraw[];
    const CellSmem s = cell_smem(smraw);
    const unsigned cnt = count[blockIdx.x];
    if (cnt == 0 || cnt > (unsigned)kCellMax) return;
    const unsigned P = (cnt + 31u) & ~31u;
    const unsigned s0 = start[blockIdx.x];
    const float qnan = __int_as_float(0x7fc00000);
    for (unsigned j = threadIdx.x; j < P; j += blockDim.x) {
        if (j < cnt) {
            uint32_t id = perm[s0 + j];
            float4 p = a[id];
            s.X[j] = p.x; s.Y[j] = p.y; s.Z[j] = p.z; s.ID[j] = id;
        } else {
            s.X[j] = qnan; s.Y[j] = qnan; s.Z[j] = qnan; s.ID[j] = kDummy;
        }
    }
    __syncthreads();
    cell_kd_sort(s, cnt);
    const unsigned o = pstart[blockIdx.x];
    for (unsigned j = threadIdx.x; j < P; j += blockDim.x) out[o + j] = s.ID[j];
}

// records in the padded k-d order; dummies get a NaN position (their w lane keeps the tag)
__global__ void k_permute4_pad(const float4* __restrict__ src, const uint32_t* __restrict__ perm, float4* __restrict__ dst,
                               uint64_t n) {
    const float qnan = __int_as_float(0x7fc00000);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t p = perm[i];
        dst[i] = p == kDummy ? make_float4(qnan, qnan, qnan, __uint_as_float(kDummy)) : src[p];
    }
}

__global__ void k_permute_u32_pad(const uint32_t* __restrict__ src, const uint32_t* __restrict__ perm,
                                  uint32_t* __restrict__ dst, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t p = perm[i];
        dst[i] = p == kDummy ? kDummy : src[p];
    }
}

// ------------------------------------------------------------------------------------------
// Exact left-balanced k-d order by streaming partitions (the photon-map build).
// Global levels 0..D-1 (nodes larger than one CTA's cell) each take these passes over
// X = float4(x, y, z, record id) in position order (and Q, each record's 16-bit coordinate):
//   hist1: per node, 256-bin histogram of the top byte of a 16-bit coordinate quantised
//          on the node's widest axis (level 0 from X; every later level gets it from the
//          split above, which also writes the coordinates to Q);
//   hist2: per node, 256-bin histogram of the low byte inside the bucket that holds the
//          cut (the node's left child takes exactly its power-of-two leaf count), from Q;
//   split: every record goes left or right of that cut (ties at the 16-bit cut resolved
//          by an atomic ticket), with warp-aggregated cursors, into X2, its coordinate on
//          its child's axis into Q, and the children's first histogram on the way.
// The remaining levels (nodes of <= kCellMax records) run in one CTA per node in shared
// memory (k_local_kd_full for perfect cells, k_local_kd for the rest). The cut is placed at
// 16-bit resolution.
// ------------------------------------------------------------------------------------------

// (start leaf a, leaf count c, path bits) of the depth-d node holding `leaf`
ALB_DEVICE void kd_node_path(uint64_t leaf, uint64_t L, int depth, uint64_t& a, uint64_t& c, uint32_t& path,
                             int& reached) {
    a = 0;
    c = L;
    path = 0;
    reached = 0;
    while (reached < depth && c > 1) {
        if ((c & (c - 1)) == 0) {
            // a perfect subtree of c = 2^e leaves: the remaining path is the leading bits of
            // the leaf's offset in it
            const int e = 63 - __clzll((long long)c);
            const int take = min(depth - reached, e);
            const uint64_t top = (leaf - a) >> (e - take);
            path = (path << take) | (uint32_t)top;
            a += top << (e - take);
            c = 1ull << (e - take);
            reached += take;
            return;
        }
        uint64_t left = 1ull << (63 - __clzll((long long)(c - 1)));
        if (leaf - a < left) {
            c = left;
            path = path << 1;
        } else {
            a += left;
            c -= left;
            path = (path << 1) | 1u;
        }
        ++reached;
    }
}

// node of the depth-d path: start leaf a and leaf count c (c == 0 if the path ends early)
ALB_DEVICE void kd_node_of_path(uint32_t path, uint64_t L, int depth, uint64_t& a, uint64_t& c) {
    a = 0;
    c = L;
    for (int i = depth - 1; i >= 0; --i) {
        if (c <= 1) {
            c = 0;
            return;
        }
        uint64_t left = 1ull << (63 - __clzll((long long)(c - 1)));
        if ((path >> i) & 1u) {
            a += left;
            c -= left;
        } else {
            c = left;
        }
    }
}

// Per node of a level: the widest box axis (x = axis bits, -1 for an empty extent), its low
// end and 65535 / extent, so that a record's 16-bit coordinate is one multiply.
struct LevelNodes {
    const float4* par;
};

__global__ void k_kdl_params(const unsigned* __restrict__ lo, const unsigned* __restrict__ hi, uint32_t nodes,
                             float4* par) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    const float l0 = ord2f(lo[3 * i]), l1 = ord2f(lo[3 * i + 1]), l2 = ord2f(lo[3 * i + 2]);
    const float e0 = ord2f(hi[3 * i]) - l0, e1 = ord2f(hi[3 * i + 1]) - l1, e2 = ord2f(hi[3 * i + 2]) - l2;
    int axis;
    float l, e;
    if (e0 >= e1 && e0 >= e2) { axis = 0; l = l0; e = e0; }
    else if (e1 >= e2) { axis = 1; l = l1; e = e1; }
    else { axis = 2; l = l2; e = e2; }
    if (!(e > 0.f)) axis = -1;
    par[i] = make_float4(__int_as_float(axis), l, axis >= 0 ? 65535.f / e : 0.f, 0.f);
}

ALB_DEVICE uint32_t kd_quant16(float4 p, LevelNodes nb, uint32_t path) {
    const float4 np = nb.par[path];
    const int axis = __float_as_int(np.x);
    if (axis < 0) return 0u;
    const float v = axis == 0 ? p.x : (axis == 1 ? p.y : p.z);
    return (uint32_t)fminf(fmaxf((v - np.y) * np.z, 0.f), 65535.f);
}

// warp-aggregated atomicAdd of 1 on cnt[key]; returns this lane's ticket
ALB_DEVICE unsigned agg_inc(unsigned* cnt, uint64_t key, unsigned active) {
    unsigned peers = __match_any_sync(active, key);
    int leader = __ffs(peers) - 1;
    unsigned rank = __popc(peers & lanemask_lt());
    unsigned base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(cnt, (unsigned)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + rank;
}

// Level passes run persistent blocks over contiguous record ranges (records of a node are
// contiguous, so a block meets few nodes at the upper levels, where global atomics would
// collide): per-node counters live in kSlots tagged shared-memory slots, records of nodes
// that find no slot go to global memory directly.
constexpr int kLvlThreads = 256;
constexpr int kSlots = 8;
constexpr int kHistItems = 4;
constexpr unsigned kNoTag = 0xffffffffu;

// claim the slot of `key` (path or child id); returns the slot or -1
ALB_DEVICE int slot_of(unsigned* tag, unsigned key) {
    const int sl = (int)(key & (kSlots - 1));
    unsigned t = tag[sl];
    if (t == kNoTag) {
        const unsigned old = atomicCAS(&tag[sl], kNoTag, key);
        t = (old == kNoTag) ? key : old;
    }
    return t == key ? sl : -1;
}

// Level 0's first pass: per node, 256-bin histogram of the top byte of the 16-bit
// coordinate, which goes to Q (later levels get both from the split of the level above).
__global__ void __launch_bounds__(kLvlThreads) k_kdl_hist1(const float4* __restrict__ X, uint16_t* Q, uint64_t n,
                                                           uint64_t L, int d, LevelNodes nb, unsigned* hist,
                                                           uint64_t per) {
    __shared__ unsigned tag[kSlots];
    __shared__ unsigned sh[kSlots * 256];
    for (int j = threadIdx.x; j < kSlots * 256; j += blockDim.x) sh[j] = 0u;
    if (threadIdx.x < kSlots) tag[threadIdx.x] = kNoTag;
    __syncthreads();
    const uint64_t r0 = blockIdx.x * per, r1 = min(r0 + per, n);
    // kHistItems records per thread and iteration, all loads issued before any is used:
    // the pass streams the records once, so loads in flight set its speed
    const uint64_t stride = (uint64_t)blockDim.x * kHistItems;
    for (uint64_t base0 = r0 + (threadIdx.x & ~31u); base0 < r1; base0 += stride) {
        float4 pv[kHistItems];
#pragma unroll
        for (int t = 0; t < kHistItems; ++t) {
            const uint64_t i = base0 + (uint64_t)t * blockDim.x + lane_id();
            if (i < r1) pv[t] = X[i];
        }
#pragma unroll
        for (int t = 0; t < kHistItems; ++t) {
            const uint64_t base = base0 + (uint64_t)t * blockDim.x;
            const uint64_t i = base + lane_id();
            bool act = false;
            uint32_t path = 0, h = 0;
            if (i < r1) {
                uint64_t a, c;
                int r;
                kd_node_path(i / 32, L, d, a, c, path, r);
                if (r == d && c > 1) {
                    const uint32_t q = kd_quant16(pv[t], nb, path);
                    Q[i] = (uint16_t)q;
                    act = true;
                    h = q >> 8;
                }
            }
            const unsigned am = __ballot_sync(0xffffffffu, act);
            if (am) {
                // a warp covers one 32-record leaf, so its records share one node: one slot
                // lookup per warp, then plain shared-memory atomics per record
                const int lead = __ffs(am) - 1;
                const uint32_t p0 = __shfl_sync(0xffffffffu, path, lead);
                if (__all_sync(0xffffffffu, !act || path == p0)) {
                    int sl = 0;
                    if ((int)lane_id() == lead) sl = slot_of(tag, p0);
                    sl = __shfl_sync(0xffffffffu, sl, lead);
                    if (act) {
                        if (sl >= 0) atomicAdd(&sh[sl * 256 + h], 1u);
                        else atomicAdd(hist + (uint64_t)path * 256 + h, 1u);
                    }
                } else if (act) {
                    const unsigned key = (path << 8) | h;
                    const unsigned peers = __match_any_sync(am, key);
                    if ((int)lane_id() == __ffs(peers) - 1) {
                        const int sl = slot_of(tag, path);
                        if (sl >= 0) atomicAdd(&sh[sl * 256 + h], (unsigned)__popc(peers));
                        else atomicAdd(hist + (uint64_t)path * 256 + h, (unsigned)__popc(peers));
                    }
                }
            }
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kSlots * 256; j += blockDim.x) {
        const unsigned t = tag[j >> 8];
        if (t != kNoTag && sh[j]) atomicAdd(hist + (uint64_t)t * 256 + (j & 255), sh[j]);
    }
}

// PASS 2 from the coordinate stream: per node, 256-bin histogram of the low byte of the
// 16-bit coordinates inside the bucket that holds the cut. Each thread takes 8 consecutive
// records (one 16-byte load of Q), which lie in one 32-record leaf and so in one node: one
// node lookup and one slot claim per 8 records.
__global__ void __launch_bounds__(kLvlThreads) k_kdl_hist2q(const uint16_t* __restrict__ Q, uint64_t n, uint64_t L,
                                                            int d, const uint2* __restrict__ sel, unsigned* hist,
                                                            uint64_t per) {
    __shared__ unsigned tag[kSlots];
    __shared__ unsigned sh[kSlots * 256];
    for (int j = threadIdx.x; j < kSlots * 256; j += blockDim.x) sh[j] = 0u;
    if (threadIdx.x < kSlots) tag[threadIdx.x] = kNoTag;
    __syncthreads();
    const uint64_t r0 = blockIdx.x * per, r1 = min(r0 + per, n);  // per is a multiple of 1024
    for (uint64_t i0 = r0 + (uint64_t)threadIdx.x * 8; i0 < r1; i0 += (uint64_t)blockDim.x * 8) {
        uint32_t q[8];
        if (i0 + 8 <= r1) {
            const uint4 v = *reinterpret_cast<const uint4*>(Q + i0);  // i0 % 8 == 0: 16-byte aligned
            q[0] = v.x & 0xffffu; q[1] = v.x >> 16; q[2] = v.y & 0xffffu; q[3] = v.y >> 16;
            q[4] = v.z & 0xffffu; q[5] = v.z >> 16; q[6] = v.w & 0xffffu; q[7] = v.w >> 16;
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) q[e] = i0 + e < r1 ? (uint32_t)Q[i0 + e] : 0u;
        }
        uint64_t a, c;
        uint32_t path;
        int r;
        kd_node_path(i0 / 32, L, d, a, c, path, r);
        if (r != d || c <= 1) continue;  // no split of this node at this level
        const unsigned bucket = sel[path].x;
        const int sl = slot_of(tag, path);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            if (i0 + e < r1 && (q[e] >> 8) == bucket) {
                if (sl >= 0) atomicAdd(&sh[sl * 256 + (q[e] & 255u)], 1u);
                else atomicAdd(hist + (uint64_t)path * 256 + (q[e] & 255u), 1u);
            }
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kSlots * 256; j += blockDim.x) {
        const unsigned t = tag[j >> 8];
        if (t != kNoTag && sh[j]) atomicAdd(hist + (uint64_t)t * 256 + (j & 255), sh[j]);
    }
}

// one warp per node: locate the bucket of the cut; sel[node] = {bucket, need inside it}
__global__ void k_kdl_select1(const unsigned* __restrict__ hist1, uint64_t L, int d, uint32_t nodes, uint2* sel) {
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int l = lane_id();
    if (w >= nodes) return;
    uint64_t a, c;
    kd_node_of_path(w, L, d, a, c);
    if (c <= 1) {
        if (l == 0) sel[w] = make_uint2(0xffffffffu, 0u);
        return;
    }
    uint64_t left = 1ull << (63 - __clzll((long long)(c - 1)));
    unsigned need = (unsigned)(left * 32);
    const unsigned* h = hist1 + (uint64_t)w * 256;
    unsigned v[8], run = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        v[j] = h[l * 8 + j];
        run += v[j];
    }
    unsigned incl = run;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (l >= o) incl += t;
    }
    unsigned before = incl - run;
    int bucket = -1;
    unsigned below = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (bucket < 0 && before < need && before + v[j] >= need) {
            bucket = l * 8 + j;
            below = before;
        }
        before += v[j];
    }
    // the node holds need + (right child's records) > need records, so one lane finds it
    unsigned who = __ballot_sync(0xffffffffu, bucket >= 0);
    int src = who ? __ffs(who) - 1 : 0;
    bucket = __shfl_sync(0xffffffffu, bucket, src);
    below = __shfl_sync(0xffffffffu, below, src);
    if (l == 0) sel[w] = make_uint2((unsigned)bucket, need - below);
}

// one warp per node: the 16-bit cut value and how many records AT it go left
__global__ void k_kdl_select2(const unsigned* __restrict__ hist2, uint32_t nodes, const uint2* __restrict__ sel,
                              uint2* cut) {
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int l = lane_id();
    if (w >= nodes) return;
    uint2 s = sel[w];
    if (s.x >= 256u) {  // not an internal node of this level
        if (l == 0) cut[w] = make_uint2(0xffffffffu, 0u);
        return;
    }
    unsigned need = s.y;
    const unsigned* h = hist2 + (uint64_t)w * 256;
    unsigned v[8], run = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        v[j] = h[l * 8 + j];
        run += v[j];
    }
    unsigned incl = run;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (l >= o) incl += t;
    }
    unsigned before = incl - run;
    int sub = -1;
    unsigned below = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (sub < 0 && before < need && before + v[j] >= need) {
            sub = l * 8 + j;
            below = before;
        }
        before += v[j];
    }
    unsigned who = __ballot_sync(0xffffffffu, sub >= 0);
    int src = who ? __ffs(who) - 1 : 0;
    sub = __shfl_sync(0xffffffffu, sub, src);
    below = __shfl_sync(0xffffffffu, below, src);
    // records with q16 < cutv go left, records with q16 == cutv: the first `ties` go left
    if (l == 0) cut[w] = make_uint2((s.x << 8) | (unsigned)(sub < 0 ? 0 : sub), need - below);
}

// Every record goes left or right of its node's cut into X2. A tile of kSplitItems records
// per thread is read once; per tile, shared counters per (node slot, side) give each record
// its rank and one global atomic per (node, side) reserves the tile's range. The children's
// boxes (for the next level's axis choice) are reduced in shared memory over the block's
// whole range and flushed once.
constexpr int kSplitItems = 4;
constexpr uint32_t kNoQ = 0xffffffffu;

__global__ void __launch_bounds__(kLvlThreads, 4) k_kdl_split(const float4* __restrict__ X, float4* __restrict__ X2,
                                                           uint16_t* Q, uint64_t n, uint64_t L, int d, LevelNodes nb,
                                                           const uint2* __restrict__ cut, unsigned* cursors,
                                                           unsigned* ties, unsigned* err, uint64_t per,
                                                           LevelNodes nbn, unsigned* hist_next) {
    __shared__ unsigned ntag[kSlots];           // node slots of the current tile
    __shared__ unsigned ncnt[kSlots * 2];       // records per (slot, side) in the tile
    __shared__ unsigned nbase[kSlots * 2];      // their global start (cursor reservation)
    // next level's first histogram (top byte of the child's 16-bit coordinate), fused into
    // this pass: child slots for the block's whole range, global counters otherwise
    __shared__ unsigned htag[kSlots];
    __shared__ unsigned hsh[kSlots * 256];
    if (hist_next) {
        for (int j = threadIdx.x; j < kSlots * 256; j += blockDim.x) hsh[j] = 0u;
        if (threadIdx.x < kSlots) htag[threadIdx.x] = kNoTag;
    }
    __syncthreads();  // the slots are read by every thread, whatever the block's range holds
    const uint64_t r0 = blockIdx.x * per, r1 = min(r0 + per, n);
    const uint64_t tile = (uint64_t)kSplitItems * blockDim.x;
    // this thread's last node lookup: leaves [cn_a, cn_a + cn_c), its path, depth reached,
    // cut and parameters
    uint64_t cn_a = 0, cn_c = 0;
    uint32_t cn_path = 0;
    int cn_r = -1;
    uint2 cn_cut = make_uint2(0u, 0u);
    float4 cn_par = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint64_t t0 = r0; t0 < r1; t0 += tile) {
        if (threadIdx.x < kSlots) ntag[threadIdx.x] = kNoTag;
        if (threadIdx.x < kSlots * 2) ncnt[threadIdx.x] = 0u;
        __syncthreads();
        float4 p[kSplitItems];
        uint64_t dst0[kSplitItems];  // start of the record's child range
        uint64_t dend[kSplitItems];  // end of that range (bounds check)
        uint32_t path[kSplitItems], rank[kSplitItems];
        uint32_t qn[kSplitItems];    // the child's 16-bit coordinate, or kNoQ when not split again
        int code[kSplitItems];       // slot * 2 + side while the tile reservation is pending, else -1
#pragma unroll
        for (int t = 0; t < kSplitItems; ++t) {  // every load in flight before the first use
            const uint64_t i = t0 + (uint64_t)t * blockDim.x + threadIdx.x;
            if (i < r1) p[t] = X[i];
        }
#pragma unroll
        for (int t = 0; t < kSplitItems; ++t) {
            const uint64_t i = t0 + (uint64_t)t * blockDim.x + threadIdx.x;
            code[t] = -1;
            dst0[t] = 0;
            dend[t] = 0;
            path[t] = 0;
            rank[t] = 0;
            qn[t] = kNoQ;
            bool moves = false, counts_next = false;
            unsigned side = 0, hbin = 0;
            uint64_t a = 0, c = 0, left = 0;
            if (i < r1) {
                // the node of the previous item usually holds this one too (items are 8
                // leaves apart, split nodes at least 128 leaves wide): reuse its lookup
                const uint64_t leaf = i / 32;
                if (!(leaf >= cn_a && leaf - cn_a < cn_c)) {
                    kd_node_path(leaf, L, d, cn_a, cn_c, cn_path, cn_r);
                    if (cn_r == d && cn_c > 1) {
                        cn_cut = cut[cn_path];
                        cn_par = nb.par[cn_path];
                    }
                }
                a = cn_a;
                c = cn_c;
                path[t] = cn_path;
                if (cn_r == d && c > 1) {
                    moves = true;
                    left = 1ull << (63 - __clzll((long long)(c - 1)));
                    const uint2 ct = cn_cut;
                    const int axis = __float_as_int(cn_par.x);
                    const float v = axis == 0 ? p[t].x : (axis == 1 ? p[t].y : p[t].z);
                    const uint32_t q = axis < 0 ? 0u : (uint32_t)fminf(fmaxf((v - cn_par.y) * cn_par.z, 0.f), 65535.f);
                    if (q < ct.x) side = 0;
                    else if (q > ct.x) side = 1;
                    else side = (atomicAdd(ties + path[t], 1u) < ct.y) ? 0u : 1u;
                    dst0[t] = a * 32 + (side ? left * 32 : 0);
                    dend[t] = side ? min((a + c) * 32, n) : (a + left) * 32;
                    // the child node is split again at the next level if it has > 1 leaf
                    if (hist_next && (side ? c - left : left) > 1) {
                        counts_next = true;
                        qn[t] = kd_quant16(p[t], nbn, (path[t] << 1) | side);
                        hbin = qn[t] >> 8;
                    }
                } else {
                    X2[i] = p[t];  // already in place (a leaf of an earlier level)
                }
            }
            // per-warp aggregation of (path, side) for the tile counters
            const unsigned am = __ballot_sync(0xffffffffu, moves);
            // a warp covers one 32-record leaf, so its moving records share one node and the
            // peers of a record are the lanes on its side (match only as a fallback)
            const unsigned right = __ballot_sync(0xffffffffu, moves && side);
            const uint32_t p0 = __shfl_sync(0xffffffffu, path[t], am ? __ffs(am) - 1 : 0);
            const bool one_node = __all_sync(0xffffffffu, !moves || path[t] == p0);
            if (moves) {
                const unsigned key = (path[t] << 1) | side;
                const unsigned peers = one_node ? (side ? right : (am & ~right)) : __match_any_sync(am, key);
                const int leader = __ffs(peers) - 1;
                const unsigned lrank = __popc(peers & lanemask_lt());
                unsigned b = 0;
                int cd = -1;
                if ((int)lane_id() == leader) {
                    const int sl = slot_of(ntag, path[t]);
                    if (sl >= 0) {
                        cd = sl * 2 + (int)side;
                        b = atomicAdd(&ncnt[cd], (unsigned)__popc(peers));
                    } else {
                        b = atomicAdd(cursors + 2 * (uint64_t)path[t] + side, (unsigned)__popc(peers));
                    }
                }
                cd = __shfl_sync(peers, cd, leader);
                b = __shfl_sync(peers, b, leader);
                code[t] = cd;
                rank[t] = b + lrank;
                if (cd < 0) {  // global cursor: final position known now
                    const uint64_t dst = dst0[t] + rank[t];
                    if (dst < dend[t]) {
                        X2[dst] = p[t];
                        if (qn[t] != kNoQ) Q[dst] = (uint16_t)qn[t];
                    } else {
                        atomicOr(err, 1u);
                    }
                }
            }
            if (counts_next) {
                const unsigned child = (path[t] << 1) | side;
                const int hs = slot_of(htag, child);
                if (hs >= 0) atomicAdd(&hsh[hs * 256 + hbin], 1u);
                else atomicAdd(hist_next + (uint64_t)child * 256 + hbin, 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x < kSlots * 2) {
            const unsigned tg = ntag[threadIdx.x >> 1];
            const unsigned cntv = ncnt[threadIdx.x];
            nbase[threadIdx.x] = (tg != kNoTag && cntv) ? atomicAdd(cursors + 2 * (uint64_t)tg + (threadIdx.x & 1), cntv) : 0u;
        }
        __syncthreads();
#pragma unroll
        for (int t = 0; t < kSplitItems; ++t) {
            if (code[t] >= 0) {
                const uint64_t dst = dst0[t] + nbase[code[t]] + rank[t];
                if (dst < dend[t]) {
                    X2[dst] = p[t];
                    if (qn[t] != kNoQ) Q[dst] = (uint16_t)qn[t];
                } else {
                    atomicOr(err, 1u);
                }
            }
        }
        __syncthreads();
    }
    if (hist_next) {
        for (int j = threadIdx.x; j < kSlots * 256; j += blockDim.x) {
            const unsigned tg = htag[j >> 8];
            if (tg != kNoTag && hsh[j]) atomicAdd(hist_next + (uint64_t)tg * 256 + (j & 255), hsh[j]);
        }
    }
}

// Children's boxes of a level: the parent's box cut on its split axis at the cut value,
// left [lo, lo + (cut + 1) / scale], right [lo + cut / scale, hi] (they overlap by one
// quantisation step). Only the next level's axis and quantisation come from these boxes;
// any box that holds the records gives the same exact median split, and the gather's box
// tree is built from the final leaves.
__global__ void k_kdl_child_boxes(const unsigned* __restrict__ lo, const unsigned* __restrict__ hi,
                                  const float4* __restrict__ par, const uint2* __restrict__ cut, uint32_t nodes,
                                  unsigned* clo, unsigned* chi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    unsigned l[3], h[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        l[k] = lo[3 * i + k];
        h[k] = hi[3 * i + k];
    }
    unsigned ll[3] = {l[0], l[1], l[2]}, lh[3] = {h[0], h[1], h[2]};
    unsigned rl[3] = {l[0], l[1], l[2]}, rh[3] = {h[0], h[1], h[2]};
    const float4 np = par[i];
    const int axis = __float_as_int(np.x);
    if (axis >= 0 && axis < 3 && np.z > 0.f) {
        const float q = (float)cut[i].x;
        const unsigned split_hi = f2ord(np.y + (q + 1.f) / np.z);
        const unsigned split_lo = f2ord(np.y + q / np.z);
        lh[axis] = min(h[axis], max(l[axis], split_hi));
        rl[axis] = max(l[axis], min(h[axis], split_lo));
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        clo[3 * (2 * (uint64_t)i) + k] = ll[k];
        chi[3 * (2 * (uint64_t)i) + k] = lh[k];
        clo[3 * (2 * (uint64_t)i + 1) + k] = rl[k];
        chi[3 * (2 * (uint64_t)i + 1) + k] = rh[k];
    }
}

// One node of <= kCellMax records X[start + j] (id in .w) per CTA, reordered in place into
// its exact left-balanced k-d order (the CTA holds the whole node in shared memory).
__global__ void __launch_bounds__(kCellThreads) k_local_kd(float4* X, const unsigned* __restrict__ cstart,
                                                           const unsigned* __restrict__ ccount, unsigned* err) {
    extern __shared__ unsigned char smraw[];
    const CellSmem s = cell_smem(smraw);
    const unsigned cnt = ccount[blockIdx.x];
    const unsigned s0 = cstart[blockIdx.x];
    if (cnt == 0) return;
    if (cnt > (unsigned)kCellMax) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        return;
    }
    const unsigned P = (cnt + 31u) & ~31u;
    const float qnan = __int_as_float(0x7fc00000);
    for (unsigned j = threadIdx.x; j < P; j += blockDim.x) {
        if (j < cnt) {
            float4 p = X[s0 + j];
            s.X[j] = p.x; s.Y[j] = p.y; s.Z[j] = p.z; s.ID[j] = __float_as_uint(p.w);
        } else {
            s.X[j] = qnan; s.Y[j] = qnan; s.Z[j] = qnan; s.ID[j] = kDummy;
        }
    }
    __syncthreads();
    cell_kd_sort(s, cnt);
    for (unsigned j = threadIdx.x; j < cnt; j += blockDim.x)
        X[s0 + j] = make_float4(s.X[j], s.Y[j], s.Z[j], __uint_as_float(s.ID[j]));
}

// Full cells (perfect subtrees of 32, 64 or 128 whole leaves: 1024, 2048 or 4096 records,
// the bulk of every large map; which size a map's cells take depends on its leaf count): the
// same k-d order as k_local_kd, with the sort keys (16-bit coordinate : 13-bit slot) held in
// registers, 8 consecutive per thread. Levels of nodes of at least kPartitionMin records are
// split by a radix partition; below it a bitonic sort runs with strides under 8 inside a
// thread, 8..128 in warp shuffles and 256 or more through shared memory; node boxes come
// from segmented warp reductions.
constexpr int kFullCell = 4096;  // the largest full cell (kCellMax)
// levels whose nodes hold at least this many records are split by a radix partition, the
// smaller ones by a bitonic sort inside a warp
constexpr unsigned kPartitionMin = 512;

template <int CELL>
struct FullCellSmem {
    float X[CELL], Y[CELL], Z[CELL];
    uint32_t ID[CELL];
    uint32_t sk[CELL];
    unsigned blo[3 * 64], bhi[3 * 64];
};

// Bitonic compare-exchange of a thread's 8 consecutive keys at a stride JJ < 8 (partners in
// the same thread; a compile-time stride keeps the keys in registers).
template <int JJ>
ALB_DEVICE void exchange_in_thread(uint32_t (&key)[8], int t, unsigned kk, unsigned S) {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        if ((e & JJ) == 0) {
            const int f = e | JJ;
            const unsigned i = (unsigned)(t * 8 + e);
            const bool up = kk == S || (i & kk) == 0;
            const uint32_t a = key[e], b = key[f];
            if ((a > b) == up) {
                key[e] = b;
                key[f] = a;
            }
        }
    }
}

// One warp: the bin of the need-th (1-based) entry of a 256-bin histogram h; need becomes the
// entry's rank inside that bin.
ALB_DEVICE unsigned pick_bin256(const uint32_t* h, unsigned& need) {
    const int lane = threadIdx.x & 31;
    uint32_t c[8], run = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        c[i] = h[lane * 8 + i];
        run += c[i];
    }
    uint32_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    uint32_t before = inc - run;
    int bin = -1;
    uint32_t below = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (bin < 0 && before + c[i] >= need) {
            bin = lane * 8 + i;
            below = before;
        }
        before += c[i];
    }
    const unsigned who = __ballot_sync(0xffffffffu, bin >= 0);
    const int src = __ffs(who) - 1;
    bin = __shfl_sync(0xffffffffu, bin, src);
    below = __shfl_sync(0xffffffffu, below, src);
    need -= below;
    return (unsigned)bin;
}

// Exclusive prefix of v over the threads of this thread's node (an aligned block of tpn >= 64
// threads, whole warps), in thread order. wsum: 16 words of shared scratch.
ALB_DEVICE unsigned node_exclusive_scan(unsigned v, uint32_t* wsum, unsigned tpn) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    unsigned inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    const int w0 = (int)((t / tpn) * (tpn / 32));
    unsigned before = 0;
    for (int i = w0; i < w; ++i) before += wsum[i];
    __syncthreads();  // wsum is reused by the next scan
    return before + inc - v;
}

template <int CELL>
__global__ void __launch_bounds__(CELL / 8, 8192 / CELL) k_local_kd_full(float4* Xg, const unsigned* __restrict__ cstart) {
    constexpr int kFullThreads = CELL / 8;
    constexpr int kLevels = CELL == 4096 ? 7 : (CELL == 2048 ? 6 : 5);  // log2(CELL / 32)
    extern __shared__ unsigned char smraw[];
    FullCellSmem<CELL>& s = *reinterpret_cast<FullCellSmem<CELL>*>(smraw);
    const uint64_t s0 = cstart[blockIdx.x];
    const int t = threadIdx.x;
    const int lane = t & 31;
    for (int j = t; j < CELL; j += kFullThreads) {
        const float4 p = Xg[s0 + j];
        s.X[j] = p.x;
        s.Y[j] = p.y;
        s.Z[j] = p.z;
        s.ID[j] = __float_as_uint(p.w);
    }
    for (int d = 0; d < kLevels; ++d) {
        const unsigned S = (unsigned)CELL >> d;  // records per node at this level
        for (int i = t; i < 3 * 64; i += kFullThreads) {
            s.blo[i] = 0xffffffffu;
            s.bhi[i] = 0u;
        }
        __syncthreads();
        // node boxes: this thread's 8 records, then the node's lanes
        unsigned mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int j = t * 8 + e;
            const unsigned o[3] = {f2ord(s.X[j]), f2ord(s.Y[j]), f2ord(s.Z[j])};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                mn[k] = min(mn[k], o[k]);
                mx[k] = max(mx[k], o[k]);
            }
        }
        const int G = S >= 256 ? 32 : (int)(S >> 3);  // lanes per node within a warp
        for (int o = 1; o < G; o <<= 1) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
                mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
            }
        }
        const unsigned node = (unsigned)(t * 8) / S;
        if ((lane & (G - 1)) == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                atomicMin(&s.blo[3 * node + k], mn[k]);
                atomicMax(&s.bhi[3 * node + k], mx[k]);
            }
        }
        __syncthreads();
        // keys: 16-bit coordinate on the node's widest axis, then the slot
        const float l0 = ord2f(s.blo[3 * node]), l1 = ord2f(s.blo[3 * node + 1]), l2 = ord2f(s.blo[3 * node + 2]);
        const float e0 = ord2f(s.bhi[3 * node]) - l0, e1 = ord2f(s.bhi[3 * node + 1]) - l1,
                    e2 = ord2f(s.bhi[3 * node + 2]) - l2;
        const int axis = (e0 >= e1 && e0 >= e2) ? 0 : (e1 >= e2 ? 1 : 2);
        const float lo = axis == 0 ? l0 : (axis == 1 ? l1 : l2);
        const float ext = axis == 0 ? e0 : (axis == 1 ? e1 : e2);
        const float* V = axis == 0 ? s.X : (axis == 1 ? s.Y : s.Z);
        uint32_t key[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int j = t * 8 + e;
            uint32_t q = 0;
            if (ext > 0.f) q = (uint32_t)fminf(fmaxf((V[j] - lo) / ext * 65535.f, 0.f), 65535.f);
            key[e] = (q << 13) | (uint32_t)j;
        }
        if (S >= kPartitionMin) {
            // Radix partition: the node's first half takes the S/2 records of smallest
            // (coordinate, position) key, the same set a sort of the keys puts there, in
            // position order; the second half the others. Two 256-bin histogram passes find
            // the cut coordinate; records AT the cut go left in position order until the left
            // half is full.
            const unsigned nodes = (unsigned)CELL / S, tpn = S / 8, nstart = node * S;
            uint32_t* h1 = s.sk;              // nodes x 256 (nodes <= CELL / 512)
            uint32_t* h2 = s.sk + CELL / 2;   // nodes x 256
            uint32_t* sel = s.blo;        // per node: cut, records at the cut that go left
            uint32_t* wsum = s.bhi;       // scan scratch (the boxes are consumed)
            for (int i = t; i < (int)(nodes * 256); i += kFullThreads) {
                h1[i] = 0u;
                h2[i] = 0u;
            }
            __syncthreads();
#pragma unroll
            for (int e = 0; e < 8; ++e) atomicAdd(&h1[node * 256 + (key[e] >> 21)], 1u);
            __syncthreads();
            const int w = t >> 5;
            if (w < (int)nodes) {
                unsigned need = S / 2;
                const unsigned b = pick_bin256(h1 + w * 256, need);
                if (lane == 0) {
                    sel[2 * w] = b;
                    sel[2 * w + 1] = need;
                }
            }
            __syncthreads();
            const unsigned hb = sel[2 * node];
#pragma unroll
            for (int e = 0; e < 8; ++e)
                if ((key[e] >> 21) == hb) atomicAdd(&h2[node * 256 + ((key[e] >> 13) & 255u)], 1u);
            __syncthreads();
            if (w < (int)nodes) {
                unsigned need = sel[2 * w + 1];
                const unsigned lb = pick_bin256(h2 + w * 256, need);
                __syncwarp();
                if (lane == 0) {
                    sel[2 * w] = (sel[2 * w] << 8) | lb;
                    sel[2 * w + 1] = need;
                }
            }
            __syncthreads();
            const unsigned cut = sel[2 * node], at_left = sel[2 * node + 1];
            unsigned nt = 0;
#pragma unroll
            for (int e = 0; e < 8; ++e) nt += (key[e] >> 13) == cut ? 1u : 0u;
            unsigned tr = node_exclusive_scan(nt, wsum, tpn);  // ties before this thread's
            unsigned lmask = 0u;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const unsigned qe = key[e] >> 13;
                bool left = qe < cut;
                if (qe == cut) left = tr++ < at_left;
                lmask |= (left ? 1u : 0u) << e;
            }
            unsigned lb4 = node_exclusive_scan((unsigned)__popc(lmask), wsum, tpn);  // lefts before
            float rx[8], ry[8], rz[8];
            uint32_t rid[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int j = t * 8 + e;
                rx[e] = s.X[j];
                ry[e] = s.Y[j];
                rz[e] = s.Z[j];
                rid[e] = s.ID[j];
            }
            __syncthreads();
            const unsigned pos0 = (unsigned)(t * 8) - nstart;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const bool left = (lmask >> e) & 1u;
                const unsigned dst = left ? nstart + lb4 : nstart + S / 2 + (pos0 + (unsigned)e - lb4);
                lb4 += left ? 1u : 0u;
                s.X[dst] = rx[e];
                s.Y[dst] = ry[e];
                s.Z[dst] = rz[e];
                s.ID[dst] = rid[e];
            }
            __syncthreads();
            continue;
        }
        // bitonic sort of every node's block of S keys, ascending
        for (unsigned kk = 2; kk <= S; kk <<= 1) {
            for (unsigned jj = kk >> 1; jj > 0; jj >>= 1) {
                if (jj >= 256) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) s.sk[t * 8 + e] = key[e];
                    __syncthreads();
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const unsigned i = (unsigned)(t * 8 + e);
                        const uint32_t o = s.sk[i ^ jj];
                        const bool lower = (i & jj) == 0, up = kk == S || (i & kk) == 0;
                        key[e] = (lower == up) ? min(key[e], o) : max(key[e], o);
                    }
                    __syncthreads();
                } else if (jj >= 8) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const unsigned i = (unsigned)(t * 8 + e);
                        const uint32_t o = __shfl_xor_sync(0xffffffffu, key[e], (int)(jj >> 3));
                        const bool lower = (i & jj) == 0, up = kk == S || (i & kk) == 0;
                        key[e] = (lower == up) ? min(key[e], o) : max(key[e], o);
                    }
                } else if (jj == 4) {
                    exchange_in_thread<4>(key, t, kk, S);
                } else if (jj == 2) {
                    exchange_in_thread<2>(key, t, kk, S);
                } else {
                    exchange_in_thread<1>(key, t, kk, S);
                }
            }
        }
        // reorder the records by the sorted slots
        float rx[8], ry[8], rz[8];
        uint32_t rid[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const uint32_t src = key[e] & 0x1fffu;
            rx[e] = s.X[src];
            ry[e] = s.Y[src];
            rz[e] = s.Z[src];
            rid[e] = s.ID[src];
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int j = t * 8 + e;
            s.X[j] = rx[e];
            s.Y[j] = ry[e];
            s.Z[j] = rz[e];
            s.ID[j] = rid[e];
        }
        __syncthreads();
    }
    for (int j = t; j < CELL; j += kFullThreads)
        Xg[s0 + j] = make_float4(s.X[j], s.Y[j], s.Z[j], __uint_as_float(s.ID[j]));
}

// positions of the interleaved store (stride 2) with each record's index in the w lane
__global__ void k_pack_ids(const float4* __restrict__ a, uint64_t n, float4* X) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float4 p = a[2 * i];
        X[i] = make_float4(p.x, p.y, p.z, __uint_as_float((uint32_t)i));
    }
}

// nodes of depth D (or leaves above it): perfect cells of 128, 64 or 32 whole leaves go to
// full[0], full[1] or full[2], the rest to (st, ct)
static void enumerate_cells(uint64_t a, uint64_t c, int depth, int D, uint64_t n, std::vector<unsigned> (&full)[3],
                            std::vector<unsigned>& st, std::vector<unsigned>& ct) {
    if (depth == D || c <= 1) {
        uint64_t s = a * 32, e = std::min<uint64_t>((a + c) * 32, n);
        const int fi = c == 128 ? 0 : (c == 64 ? 1 : (c == 32 ? 2 : -1));
        if (fi >= 0 && e - s == c * 32) {
            full[fi].push_back((unsigned)s);
        } else if (e > s) {
            st.push_back((unsigned)s);
            ct.push_back((unsigned)(e - s));
        }
        return;
    }
    uint64_t left = 1ull << (63 - __builtin_clzll((unsigned long long)(c - 1)));
    enumerate_cells(a, left, depth + 1, D, n, full, st, ct);
    enumerate_cells(a + left, c - left, depth + 1, D, n, full, st, ct);
}

// out[i] <- (position, record id) of the i-th record of `a` (the interleaved record store:
// record i at a[2 i]) in exact left-balanced k-d order.
// `out` (n float4) is one of the two ping-pong buffers, so the build needs one temporary of
// the same size besides it.
static int kd_order_fast(Workspace& ws, const float4* a, uint64_t n, const float blo[3], const float bhi[3],
                         float4* out, cudaStream_t st) {
    const uint64_t L = (n + 31) / 32;
    int depth_max = L > 1 ? 64 - __builtin_clzll((unsigned long long)(L - 1)) : 0;
    const int local_levels = 7;  // kCellMax / 32 = 128 leaves = 2^7
    const int D = std::max(0, depth_max - local_levels);
    size_t mark = ws.mark();
    float4* tmp = (float4*)ws.take_bytes(n * 16);
    unsigned* err = ws.take_u32(1);
    if (!tmp || !err) {
        ws.release(mark);
        return -1;
    }
    // D partition levels swap the buffers D times: start so that the result lands in `out`
    float4* X = (D % 2 == 0) ? out : tmp;
    float4* X2 = (D % 2 == 0) ? tmp : out;
    cudaMemsetAsync(err, 0, 4, st);
    unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 16384);
    k_pack_ids<<<blocks, 256, 0, st>>>(a, n, X);
    note_launch();
    if (D > 0) {
        const uint64_t maxnodes = 1ull << D;
        unsigned* hist1 = ws.take_u32(maxnodes * 256);
        unsigned* hist2 = ws.take_u32(maxnodes * 256);
        uint2* sel = (uint2*)ws.take_bytes(maxnodes * 8);
        uint2* cut = (uint2*)ws.take_bytes(maxnodes * 8);
        unsigned* cursors = ws.take_u32(maxnodes * 2);
        unsigned* ties = ws.take_u32(maxnodes);
        unsigned* lo = ws.take_u32(maxnodes * 6);  // current level boxes
        unsigned* hi = ws.take_u32(maxnodes * 6);
        unsigned* clo = ws.take_u32(maxnodes * 6);  // children boxes
        unsigned* chi = ws.take_u32(maxnodes * 6);
        float4* par = (float4*)ws.take_bytes(maxnodes * 16);
        float4* cpar = (float4*)ws.take_bytes(maxnodes * 16);  // children's parameters
        unsigned* hist1n = ws.take_u32(maxnodes * 256);       // children's first histogram
        // each record's 16-bit coordinate on its node's axis, in position order: written by
        // the level-0 histogram and by every split for the next level, read by the second
        // histogram instead of the whole record
        uint16_t* Q = (uint16_t*)ws.take_bytes(n * 2);
        if (!hist1 || !hist2 || !sel || !cut || !cursors || !ties || !lo || !hi || !clo || !chi || !par || !cpar ||
            !hist1n || !Q) {
            ws.release(mark);
            return -1;
        }
        // level 0 box: the records' bounding box
        unsigned h6[6];
        for (int k = 0; k < 3; ++k) {
            uint32_t u;
            memcpy(&u, &blo[k], 4);
            h6[k] = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
            memcpy(&u, &bhi[k], 4);
            h6[3 + k] = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        }
        unsigned init_lo[3] = {h6[0], h6[1], h6[2]}, init_hi[3] = {h6[3], h6[4], h6[5]};
        cudaMemcpyAsync(lo, init_lo, 12, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(hi, init_hi, 12, cudaMemcpyHostToDevice, st);
        // persistent level blocks over contiguous ranges (a multiple of the split tile)
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const uint64_t lvl_blocks = std::max<uint64_t>(1, std::min<uint64_t>((n + 4095) / 4096, (uint64_t)sms * 8));
        uint64_t per = (n + lvl_blocks - 1) / lvl_blocks;
        per = (per + 1023) & ~1023ull;
        const unsigned lb = (unsigned)((n + per - 1) / per);
        // level 0: its parameters and first histogram; every later level gets both from
        // the previous level (children's boxes, and the histogram fused into the split pass)
        k_kdl_params<<<1, 256, 0, st>>>(lo, hi, 1u, par);
        note_launch();
        cudaMemsetAsync(hist1, 0, 256 * 4, st);
        k_kdl_hist1<<<lb, kLvlThreads, 0, st>>>(X, Q, n, L, 0, LevelNodes{par}, hist1, per);
        note_launch();
        for (int d = 0; d < D; ++d) {
            const uint32_t nodes = 1u << d;
            const bool more = d + 1 < D;
            cudaMemsetAsync(hist2, 0, (size_t)nodes * 256 * 4, st);
            cudaMemsetAsync(cursors, 0, (size_t)nodes * 8, st);
            cudaMemsetAsync(ties, 0, (size_t)nodes * 4, st);
            LevelNodes nb{par};
            k_kdl_select1<<<(nodes * 32 + 255) / 256, 256, 0, st>>>(hist1, L, d, nodes, sel);
            note_launch();
            k_kdl_hist2q<<<lb, kLvlThreads, 0, st>>>(Q, n, L, d, sel, hist2, per);
            note_launch();
            k_kdl_select2<<<(nodes * 32 + 255) / 256, 256, 0, st>>>(hist2, nodes, sel, cut);
            note_launch();
            if (more) {
                k_kdl_child_boxes<<<(nodes + 255) / 256, 256, 0, st>>>(lo, hi, par, cut, nodes, clo, chi);
                note_launch();
                k_kdl_params<<<(2 * nodes + 255) / 256, 256, 0, st>>>(clo, chi, 2 * nodes, cpar);
                note_launch();
                cudaMemsetAsync(hist1n, 0, (size_t)nodes * 2 * 256 * 4, st);
            }
            k_kdl_split<<<lb, kLvlThreads, 0, st>>>(X, X2, Q, n, L, d, nb, cut, cursors, ties, err, per,
                                                     LevelNodes{cpar}, more ? hist1n : nullptr);
            note_launch();
            std::swap(X, X2);
            std::swap(lo, clo);
            std::swap(hi, chi);
            std::swap(par, cpar);
            std::swap(hist1, hist1n);
        }
    }
    // local levels: one CTA per remaining node
    std::vector<unsigned> fs[3], cs, cc;
    enumerate_cells(0, L, 0, D, n, fs, cs, cc);
    unsigned* dfs[3];
    for (int f = 0; f < 3; ++f) dfs[f] = ws.take_u32(fs[f].size() + 1);
    unsigned* dcs = ws.take_u32(cs.size() + 1);
    unsigned* dcc = ws.take_u32(cc.size() + 1);
    if (!dfs[0] || !dfs[1] || !dfs[2] || !dcs || !dcc) {
        ws.release(mark);
        return -1;
    }
    for (int f = 0; f < 3; ++f)
        if (!fs[f].empty()) cudaMemcpyAsync(dfs[f], fs[f].data(), fs[f].size() * 4, cudaMemcpyHostToDevice, st);
    if (!cs.empty()) {
        cudaMemcpyAsync(dcs, cs.data(), cs.size() * 4, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dcc, cc.data(), cc.size() * 4, cudaMemcpyHostToDevice, st);
    }
    static std::atomic<bool> attr_set[64];  // batched runs build from several host threads
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_set[dev].load(std::memory_order_acquire)) {
        cudaFuncSetAttribute(k_local_kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cell_smem_bytes());
        cudaFuncSetAttribute(k_local_kd_full<4096>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(FullCellSmem<4096>));
        cudaFuncSetAttribute(k_local_kd_full<2048>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(FullCellSmem<2048>));
        cudaFuncSetAttribute(k_local_kd_full<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(FullCellSmem<1024>));
        attr_set[dev].store(true, std::memory_order_release);
    }
    if (!fs[0].empty()) {
        k_local_kd_full<4096><<<(unsigned)fs[0].size(), 512, sizeof(FullCellSmem<4096>), st>>>(X, dfs[0]);
        note_launch();
    }
    if (!fs[1].empty()) {
        k_local_kd_full<2048><<<(unsigned)fs[1].size(), 256, sizeof(FullCellSmem<2048>), st>>>(X, dfs[1]);
        note_launch();
    }
    if (!fs[2].empty()) {
        k_local_kd_full<1024><<<(unsigned)fs[2].size(), 128, sizeof(FullCellSmem<1024>), st>>>(X, dfs[2]);
        note_launch();
    }
    if (!cs.empty()) {
        k_local_kd<<<(unsigned)cs.size(), kCellThreads, cell_smem_bytes(), st>>>(X, dcs, dcc, err);
        note_launch();
    }
    unsigned herr = 0;
    cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);  // also keeps the host vectors alive for their copies
    ws.release(mark);
    return herr ? -1 : 0;
}

// ------------------------------------------------------------------------------------------
// permutation and box tree
// ------------------------------------------------------------------------------------------

// One warp per leaf: box of 32 consecutive sorted records.
__global__ void k_leaf_boxes(const float4* __restrict__ a, uint64_t n, float4* lo, float4* hi, uint64_t nleaf) {
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    int l = threadIdx.x & 31;
    if (warp >= nleaf) return;
    uint64_t i = warp * 32 + l;
    float x0 = 3.4e38f, y0 = 3.4e38f, z0 = 3.4e38f, x1 = -3.4e38f, y1 = -3.4e38f, z1 = -3.4e38f;
    if (i < n) {
        float4 p = a[i];
        x0 = x1 = p.x; y0 = y1 = p.y; z0 = z1 = p.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
        x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        z0 = fminf(z0, __shfl_xor_sync(0xffffffffu, z0, o));
        x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        z1 = fmaxf(z1, __shfl_xor_sync(0xffffffffu, z1, o));
    }
    if (l == 0) {
        lo[warp] = make_float4(x0, y0, z0, 0.f);
        hi[warp] = make_float4(x1, y1, z1, 0.f);
    }
}

// One warp per parent: union of up to 32 child boxes.
__global__ void k_parent_boxes(const float4* __restrict__ clo, const float4* __restrict__ chi, uint64_t nchild,
                               float4* plo, float4* phi, uint64_t nparent) {
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    int l = threadIdx.x & 31;
    if (warp >= nparent) return;
    uint64_t i = warp * 32 + l;
    float x0 = 3.4e38f, y0 = 3.4e38f, z0 = 3.4e38f, x1 = -3.4e38f, y1 = -3.4e38f, z1 = -3.4e38f;
    if (i < nchild) {
        float4 a = clo[i], b = chi[i];
        x0 = a.x; y0 = a.y; z0 = a.z; x1 = b.x; y1 = b.y; z1 = b.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
        x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        z0 = fminf(z0, __shfl_xor_sync(0xffffffffu, z0, o));
        x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        z1 = fmaxf(z1, __shfl_xor_sync(0xffffffffu, z1, o));
    }
    if (l == 0) {
        plo[warp] = make_float4(x0, y0, z0, 0.f);
        phi[warp] = make_float4(x1, y1, z1, 0.f);
    }
}

// ------------------------------------------------------------------------------------------
// host drivers
// ------------------------------------------------------------------------------------------

KeyGrid make_key_grid(const float lo[3], const float hi[3], int bits3, int bits2) {
    KeyGrid g{};
    float ext[3], emax = 0.f;
    for (int k = 0; k < 3; ++k) {
        ext[k] = hi[k] - lo[k];
        emax = std::max(emax, ext[k]);
    }
    int na = 0;
    for (int k = 0; k < 3; ++k) {
        g.lo[k] = lo[k];
        // an axis with (almost) no extent carries no key bits (planar surface/floor maps)
        if (ext[k] > 1e-6f * std::max(emax, 1e-30f) && ext[k] > 0.f) g.ax[na++] = k;
    }
    g.naxes = na;
    const int bits = na == 3 ? bits3 : bits2;
    for (int k = 0; k < 3; ++k) {
        bool active = false;
        for (int j = 0; j < na; ++j) active |= (g.ax[j] == k);
        if (!active) {
            g.scale[k] = 0.0;
            g.maxq[k] = 0.0;
            continue;
        }
        double maxq = (double)((1ull << bits) - 1ull);
        g.maxq[k] = maxq;
        g.scale[k] = maxq / (double)ext[k];
    }
    return g;
}

int build_box_tree(Workspace& ws, MapIndex& m, cudaStream_t st) {
    uint64_t n = m.n;
    uint64_t cnt = (n + 31) / 32;
    int lev = 0;
    uint64_t off = 0;
    while (true) {
        m.lvl_off[lev] = off;
        m.lvl_cnt[lev] = cnt;
        off += cnt;
        ++lev;
        if (cnt <= 32 || lev >= kMaxLevels) break;
        cnt = (cnt + 31) / 32;
    }
    m.nlevels = lev;
    m.nboxes = off;
    m.box_lo = (float4*)ws.alloc_persistent(m.box_lo, m.box_cap, off);
    m.box_hi = (float4*)ws.alloc_persistent(m.box_hi, m.box_cap_hi, off);
    if (!m.box_lo || !m.box_hi) return -1;
    uint64_t nl = m.lvl_cnt[0];
    k_leaf_boxes<<<(unsigned)((nl * 32 + 255) / 256), 256, 0, st>>>(m.a, n, m.box_lo, m.box_hi, nl);
    note_launch();
    for (int l = 1; l < m.nlevels; ++l) {
        uint64_t np = m.lvl_cnt[l];
        k_parent_boxes<<<(unsigned)((np * 32 + 255) / 256), 256, 0, st>>>(
            m.box_lo + m.lvl_off[l - 1], m.box_hi + m.lvl_off[l - 1], m.lvl_cnt[l - 1],
            m.box_lo + m.lvl_off[l], m.box_hi + m.lvl_off[l], np);
        note_launch();
    }
    return 0;
}

int compute_bbox(Workspace& ws, const float4* a, uint64_t n, float lo[3], float hi[3], cudaStream_t st,
                 uint64_t stride) {
    unsigned* box = ws.scratch_box();
    if (!box) return -1;
    unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    cudaMemcpyAsync(box, init, sizeof(init), cudaMemcpyHostToDevice, st);
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks == 0) blocks = 1;
    k_bbox<<<blocks, 256, 0, st>>>(a, stride, n, box);
    note_launch();
    unsigned h[6];
    cudaMemcpyAsync(h, box, sizeof(h), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    for (int k = 0; k < 3; ++k) {
        lo[k] = ord2f(h[k]);
        hi[k] = ord2f(h[3 + k]);
    }
    return 0;
}

// a[i] holds (position, record id) in index order: gather every record field into index
// order, a last (in place: each thread reads its id before overwriting the entry).
__global__ void k_finalize(float4* a, float4* __restrict__ b, float4* __restrict__ fwi, float4* __restrict__ sfi,
                           uint32_t* __restrict__ id, float4* __restrict__ sco, RecordStore rec, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = __float_as_uint(a[i].w);
        b[i] = rec.b[2 * (uint64_t)r];  // the record's two halves share one 32-byte sector
        if (fwi) {
            fwi[i] = rec.fwi[r];
            sfi[i] = rec.sfi[r];
        }
        if (id) id[i] = rec.id[r];
        if (sco) sco[i] = rec.sco[r];
        a[i] = rec.a[2 * (uint64_t)r];
    }
}

void release_map_index(MapIndex& m) {
    cudaFree(m.a); cudaFree(m.b); cudaFree(m.fwi); cudaFree(m.sfi); cudaFree(m.id); cudaFree(m.sco);
    m.a = m.b = m.fwi = m.sfi = m.sco = nullptr;
    m.id = nullptr;
    m.a_cap = m.b_cap = m.fwi_cap = m.sfi_cap = m.id_cap = m.sco_cap = 0;
}

// Build the k-d index of one channel's n records: records in exact left-balanced k-d order
// over 32-record leaves, plus the box tree. The previous index arrays are released first,
// so the peak is the record store plus two n-record float4 buffers.
int build_map_index(Workspace& ws, const RecordStore& rec, uint64_t n, MapIndex& m, cudaStream_t st) {
    m.n = n;
    m.n_real = n;
    if (n == 0) {
        m.nlevels = 0;
        return 0;
    }
    if (n >= (1ull << 32)) return -1;  // record ids are 32-bit
    float lo[3], hi[3];
    if (compute_bbox(ws, rec.a, n, lo, hi, st, 2) != 0) return -1;
    cudaStreamSynchronize(st);
    if (n > m.a_cap) release_map_index(m);  // else every array is reused in place
    m.a = (float4*)ws.alloc_persistent(m.a, m.a_cap, n);
    if (!m.a || kd_order_fast(ws, rec.a, n, lo, hi, m.a, st) != 0) return -1;
    cudaStreamSynchronize(st);  // the build temporary is back in the pool
    m.b = (float4*)ws.alloc_persistent(m.b, m.b_cap, n);
    if (rec.fwi) {
        m.fwi = (float4*)ws.alloc_persistent(m.fwi, m.fwi_cap, n);
        m.sfi = (float4*)ws.alloc_persistent(m.sfi, m.sfi_cap, n);
    }
    if (rec.id) m.id = (uint32_t*)ws.alloc_persistent_u32(m.id, m.id_cap, n);
    if (rec.sco) m.sco = (float4*)ws.alloc_persistent(m.sco, m.sco_cap, n);
    if (!m.b || (rec.fwi && (!m.fwi || !m.sfi)) || (rec.id && !m.id) || (rec.sco && !m.sco)) return -1;
    // one record per thread: the gathers are random, so many loads in flight matter
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_finalize<<<blocks, 256, 0, st>>>(m.a, m.b, rec.fwi ? m.fwi : nullptr, rec.fwi ? m.sfi : nullptr,
                                       rec.id ? m.id : nullptr, rec.sco ? m.sco : nullptr, rec, n);
    note_launch();
    return build_box_tree(ws, m, st);
}

// Single-cell index build into caller-provided device memory (no allocation): the k-d
// order of n <= kCellMax points (one CTA), the padded permuted copy and its box tree.
// `cell` holds {start = 0, count = n, pstart = 0}; perm_in is the identity.
int cell_index_max_points() { return kCellMax; }

void launch_single_cell_index(const float4* pts, uint32_t n, const uint32_t* perm_in, const unsigned* cell,
                              uint32_t* perm_out, float4* sorted, float4* box_lo, float4* box_hi,
                              const uint64_t* lvl_off, const uint64_t* lvl_cnt, int nlevels, cudaStream_t st) {
    static std::atomic<bool> attr_set[64];  // batched runs build from several host threads
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_set[dev].load(std::memory_order_acquire)) {
        cudaFuncSetAttribute(k_cell_kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cell_smem_bytes());
        attr_set[dev].store(true, std::memory_order_release);
    }
    const uint32_t P = (n + 31u) & ~31u;
    k_cell_kd<<<1, kCellThreads, cell_smem_bytes(), st>>>(pts, perm_in, cell, cell + 1, cell + 2, perm_out);
    note_launch();
    k_permute4_pad<<<(P + 255) / 256, 256, 0, st>>>(pts, perm_out, sorted, P);
    note_launch();
    k_leaf_boxes<<<(unsigned)((lvl_cnt[0] * 32 + 255) / 256), 256, 0, st>>>(sorted, P, box_lo, box_hi, lvl_cnt[0]);
    note_launch();
    for (int l = 1; l < nlevels; ++l) {
        k_parent_boxes<<<(unsigned)((lvl_cnt[l] * 32 + 255) / 256), 256, 0, st>>>(
            box_lo + lvl_off[l - 1], box_hi + lvl_off[l - 1], lvl_cnt[l - 1], box_lo + lvl_off[l], box_hi + lvl_off[l],
            lvl_cnt[l]);
        note_launch();
    }
}

// Spatial order of gather queries under a map's key grid (for cache locality).
// The queries are ordered along a Morton curve over their own bounding box: over the map's
// box, queries far from a compact map (surface-reflection queries around the laser spot)
// would clamp to its edge and lose their order. 10 bits per axis in 3-D and 16 in 2-D make
// cells far finer than any k-th-neighbour distance with half the radix passes of full-width
// keys; the order only steers the search bounds, never the result.
int sort_queries(Workspace& ws, const float4* qa, uint64_t n, uint32_t* perm, cudaStream_t st) {
    if (n == 0) return 0;
    float qlo[3], qhi[3];
    if (compute_bbox(ws, qa, n, qlo, qhi, st) != 0) return -1;
    const KeyGrid g = make_key_grid(qlo, qhi, 10, 16);
    size_t mark = ws.mark();
    uint32_t* keys = ws.take_u32(n);
    uint32_t* vals = perm;
    uint32_t* keys2 = ws.take_u32(n);
    uint32_t* vals2 = ws.take_u32(n);
    unsigned long long* oa = (unsigned long long*)ws.scratch_box();
    if (!keys || !keys2 || !vals2 || !oa) {  // nothing launched on a failed allocation
        ws.release(mark);
        return -1;
    }
    unsigned long long init[2] = {0ull, ~0ull};
    cudaMemcpyAsync(oa, init, sizeof(init), cudaMemcpyHostToDevice, st);
    unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 8192);
    k_keys<<<blocks, 256, 0, st>>>(qa, n, g, keys, vals, oa);
    note_launch();
    unsigned long long h[2];
    cudaMemcpyAsync(h, oa, sizeof(h), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    uint32_t* k0 = keys;
    uint32_t* v0 = vals;
    if (radix_sort_pairs<uint32_t>(ws, k0, v0, keys2, vals2, n, h[0] ^ h[1], st) < 0) {
        ws.release(mark);
        return -1;
    }
    if (v0 != perm) cudaMemcpyAsync(perm, v0, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    ws.release(mark);
    return 0;
}

}  // namespace alb
