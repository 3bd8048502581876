// Photon-map index build: the GPU replacement of build_photon_map_data + PhotonMapIndex
// (alb_sim/photon_mapping/build_photon_map_data.py:8-62, photon_map_index.py:6-17).
//
// Records are ordered along a Morton curve of a uniform grid over the map's bounding box
// (cell key = interleaved cell coordinates, 32 bits) by an LSD radix sort, permuted into
// that order as two float4 streams, and cut into buckets of 32 consecutive records. A
// bucket's bounding box is a leaf; 32 consecutive boxes form the next level up, until 32
// or fewer boxes remain. The gather walks this implicit 32-ary box tree warp-wide.
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
__global__ void k_bbox(const float4* __restrict__ a, const float4* __restrict__ c, uint64_t n,
                       unsigned* box) {
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float4 p = a[i];
        float x = p.x, y = p.y, z = p.z;
        if (c) {  // query streams carry a low part; the box only needs the float part
            (void)c;
        }
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
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(box + k, f2ord(lo[k]));
            atomicMax(box + 3 + k, f2ord(hi[k]));
        }
    }
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

__global__ void k_keys(const float4* __restrict__ a, uint64_t n, KeyGrid g, uint64_t* keys, uint32_t* vals,
                       unsigned long long* or_and) {
    unsigned long long o = 0ull, an = ~0ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float4 p = a[i];
        uint64_t key = morton_key(g, p.x, p.y, p.z);
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

static void exclusive_scan(Workspace& ws, uint32_t* data, uint64_t n, cudaStream_t st) {
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles <= 1) {
        k_scan_tile<<<1, kScanThreads, 0, st>>>(data, n, nullptr);
        note_launch();
        return;
    }
    uint32_t* sums = ws.take_u32(tiles);
    k_scan_tile<<<(unsigned)tiles, kScanThreads, 0, st>>>(data, n, sums);
    note_launch();
    exclusive_scan(ws, sums, tiles, st);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(data, n, sums);
    note_launch();
}

int radix_sort_pairs(Workspace& ws, uint64_t*& keys, uint32_t*& vals, uint64_t*& keys_alt,
                     uint32_t*& vals_alt, uint64_t n, uint64_t varying_bits, cudaStream_t st) {
    if (n <= 1) return 0;
    const uint32_t ntiles = (uint32_t)((n + kRsTile - 1) / kRsTile);
    size_t mark = ws.mark();
    uint32_t* hist = ws.take_u32((uint64_t)ntiles * 256);
    int passes = 0;
    for (int shift = 0; shift < 64; shift += 8) {
        if (((varying_bits >> shift) & 255ull) == 0ull) continue;  // digit constant over all keys
        k_rs_hist<<<ntiles, kRsThreads, 0, st>>>(keys, n, shift, hist, ntiles);
        note_launch();
        exclusive_scan(ws, hist, (uint64_t)ntiles * 256, st);
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
// Built level by level: node boxes -> key (node, 16-bit coordinate on the node's widest
// axis) -> stable radix sort of (key, permutation).
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

__global__ void k_iota(uint32_t* p, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = (uint32_t)i;
}

// node boxes of this level (ordered-int min/max), warp-aggregated when a warp is in one node
__global__ void k_kd_bbox(const float4* __restrict__ a, const uint32_t* __restrict__ perm, uint64_t n, uint64_t L,
                          int depth, unsigned* lo, unsigned* hi) {
    for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; base < n;
         base += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t i = base + (threadIdx.x & 31);
        bool valid = i < n;
        uint64_t na = 0, nc = 0;
        float x = 0.f, y = 0.f, z = 0.f;
        if (valid) {
            kd_node(i / 32, L, depth, na, nc);
            float4 p = a[perm[i]];
            x = p.x; y = p.y; z = p.z;
        }
        unsigned long long key = valid ? na : ~0ull;
        unsigned peers = __match_any_sync(0xffffffffu, key);
        unsigned ox0 = f2ord(x), oy0 = f2ord(y), oz0 = f2ord(z);
        unsigned ox1 = ox0, oy1 = oy0, oz1 = oz0;
        if (peers == 0xffffffffu) {
            for (int o = 16; o > 0; o >>= 1) {
                ox0 = min(ox0, __shfl_xor_sync(0xffffffffu, ox0, o)); ox1 = max(ox1, __shfl_xor_sync(0xffffffffu, ox1, o));
                oy0 = min(oy0, __shfl_xor_sync(0xffffffffu, oy0, o)); oy1 = max(oy1, __shfl_xor_sync(0xffffffffu, oy1, o));
                oz0 = min(oz0, __shfl_xor_sync(0xffffffffu, oz0, o)); oz1 = max(oz1, __shfl_xor_sync(0xffffffffu, oz1, o));
            }
            if ((threadIdx.x & 31) != 0) continue;
        }
        if (!valid || nc <= 1) continue;
        atomicMin(lo + 3 * na, ox0); atomicMin(lo + 3 * na + 1, oy0); atomicMin(lo + 3 * na + 2, oz0);
        atomicMax(hi + 3 * na, ox1); atomicMax(hi + 3 * na + 1, oy1); atomicMax(hi + 3 * na + 2, oz1);
    }
}

__global__ void k_kd_keys(const float4* __restrict__ a, const uint32_t* __restrict__ perm, uint64_t n, uint64_t L,
                          int depth, const unsigned* __restrict__ lo, const unsigned* __restrict__ hi, uint64_t* keys,
                          unsigned long long* or_and) {
    unsigned long long o = 0ull, an = ~0ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t na, nc;
        kd_node(i / 32, L, depth, na, nc);
        uint64_t q = 0;
        if (nc > 1) {
            float l0 = ord2f(lo[3 * na]), l1 = ord2f(lo[3 * na + 1]), l2 = ord2f(lo[3 * na + 2]);
            float e0 = ord2f(hi[3 * na]) - l0, e1 = ord2f(hi[3 * na + 1]) - l1, e2 = ord2f(hi[3 * na + 2]) - l2;
            float4 p = a[perm[i]];
            float v, l, e;
            if (e0 >= e1 && e0 >= e2) { v = p.x; l = l0; e = e0; }
            else if (e1 >= e2) { v = p.y; l = l1; e = e1; }
            else { v = p.z; l = l2; e = e2; }
            if (e > 0.f) q = (uint64_t)fminf(fmaxf((v - l) / e * 65535.f, 0.f), 65535.f);
        }
        uint64_t key = (na << 16) | q;
        keys[i] = key;
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

// perm <- k-d order of the n records of `a`
static void kd_order(Workspace& ws, const float4* a, uint64_t n, uint32_t*& perm, uint32_t*& perm_alt,
                     cudaStream_t st) {
    const uint64_t L = (n + 31) / 32;
    unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 16384);
    k_iota<<<blocks, 256, 0, st>>>(perm, n);
    note_launch();
    if (L <= 1) return;
    int depth_max = 64 - __builtin_clzll((unsigned long long)(L - 1));  // ceil(log2 L)
    size_t mark = ws.mark();
    unsigned* lo = (unsigned*)ws.take_bytes(L * 12);
    unsigned* hi = (unsigned*)ws.take_bytes(L * 12);
    uint64_t* keys = (uint64_t*)ws.take_bytes(n * 8);
    uint64_t* keys2 = (uint64_t*)ws.take_bytes(n * 8);
    unsigned long long* oa = (unsigned long long*)ws.scratch_box();
    for (int d = 0; d < depth_max; ++d) {
        cudaMemsetAsync(lo, 0xff, L * 12, st);
        cudaMemsetAsync(hi, 0x00, L * 12, st);
        k_kd_bbox<<<blocks, 256, 0, st>>>(a, perm, n, L, d, lo, hi);
        note_launch();
        unsigned long long init[2] = {0ull, ~0ull};
        cudaMemcpyAsync(oa, init, sizeof(init), cudaMemcpyHostToDevice, st);
        k_kd_keys<<<blocks, 256, 0, st>>>(a, perm, n, L, d, lo, hi, keys, oa);
        note_launch();
        unsigned long long h[2];
        cudaMemcpyAsync(h, oa, sizeof(h), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        uint64_t* k0 = keys;
        uint64_t* k1 = keys2;
        radix_sort_pairs(ws, k0, perm, k1, perm_alt, n, h[0] ^ h[1], st);
    }
    ws.release(mark);
}

// ------------------------------------------------------------------------------------------
// Sample-partitioned k-d order (the build used for photon maps):
//  1. a median-split k-d tree of T levels is built on a strided sample of the records
//     (kd_order above, on the sample only);
//  2. every record descends the T split planes to one of 2^T cells (one pass);
//  3. one radix sort groups the records by cell;
//  4. one CTA per cell finishes an exact left-balanced k-d order of the cell's records in
//     shared memory and pads the cell to whole 32-record leaves with dummy records (NaN
//     position: never admitted by the gather, ignored by the box reductions).
// Leaves therefore never straddle cells and are exact k-d leaves inside them.
// ------------------------------------------------------------------------------------------
__global__ void k_permute4(const float4* __restrict__ src, const uint32_t* __restrict__ perm,
                           float4* __restrict__ dst, uint64_t n);

constexpr int kCellMax = 4096;     // records per cell handled by one CTA
constexpr int kCellThreads = 512;
constexpr uint32_t kDummy = 0xffffffffu;

__global__ void k_take_sample(const float4* __restrict__ a, uint64_t n, uint64_t stride, uint64_t S, float4* out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < S; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t j = i * stride;
        out[i] = a[j < n ? j : n - 1];
    }
}

// split planes of the top tree (heap order, node 1 = root) from the k-d ordered sample:
// node j of level d covers sample positions [j*seg, (j+1)*seg), seg = S >> d; its plane is
// the widest axis of the node's sample box at the coordinate of the element seg/2.
// one CTA (256 threads) per node h = blockIdx.x + 1
__global__ void __launch_bounds__(256) k_top_planes(const float4* __restrict__ s, uint64_t S, uint8_t* axis, float* value) {
    __shared__ float red[6][8];
    __shared__ int ax_s;
    const uint64_t h = (uint64_t)blockIdx.x + 1;
    const int d = 63 - __clzll((long long)h);
    const uint64_t j = h - (1ull << d);
    const uint64_t seg = S >> d;
    const uint64_t b = j * seg, e = b + seg;
    float v6[6] = {3.4e38f, 3.4e38f, 3.4e38f, -3.4e38f, -3.4e38f, -3.4e38f};
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        float4 p = s[i];
        v6[0] = fminf(v6[0], p.x); v6[3] = fmaxf(v6[3], p.x);
        v6[1] = fminf(v6[1], p.y); v6[4] = fmaxf(v6[4], p.y);
        v6[2] = fminf(v6[2], p.z); v6[5] = fmaxf(v6[5], p.z);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            float x = __shfl_xor_sync(0xffffffffu, v6[k], o);
            v6[k] = k < 3 ? fminf(v6[k], x) : fmaxf(v6[k], x);
        }
        if (l == 0) red[k][w] = v6[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float r[6];
        for (int k = 0; k < 6; ++k) {
            r[k] = red[k][0];
            for (int q = 1; q < 8; ++q) r[k] = k < 3 ? fminf(r[k], red[k][q]) : fmaxf(r[k], red[k][q]);
        }
        float e0 = r[3] - r[0], e1 = r[4] - r[1], e2 = r[5] - r[2];
        ax_s = (e0 >= e1 && e0 >= e2) ? 0 : (e1 >= e2 ? 1 : 2);
    }
    __syncthreads();
    // the sample inside the node is k-d ordered with its two halves as the children, so the
    // plane is the largest coordinate of the left half on the node's axis
    const int ax = ax_s;
    float vmax = -3.4e38f;
    for (uint64_t i = b + threadIdx.x; i < b + seg / 2; i += blockDim.x) {
        float4 p = s[i];
        vmax = fmaxf(vmax, ax == 0 ? p.x : (ax == 1 ? p.y : p.z));
    }
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    __syncthreads();
    if (l == 0) red[0][w] = vmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = red[0][0];
        for (int q = 1; q < 8; ++q) r = fmaxf(r, red[0][q]);
        axis[h] = (uint8_t)ax;
        value[h] = r;
    }
}

__global__ void k_assign_cells(const float4* __restrict__ a, uint64_t n, int T, const uint8_t* __restrict__ axis,
                               const float* __restrict__ value, uint64_t* keys, uint32_t* vals, unsigned* counts) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float4 p = a[i];
        uint32_t h = 1;
        for (int d = 0; d < T; ++d) {
            int ax = axis[h];
            float c = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
            h = 2 * h + (c > value[h] ? 1u : 0u);
        }
        uint32_t cell = h - (1u << T);
        keys[i] = cell;
        vals[i] = (uint32_t)i;
        atomicAdd(counts + cell, 1u);
    }
}

__global__ void k_pad_counts(const unsigned* __restrict__ counts, uint32_t ncell, unsigned* padded, unsigned* maxc) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        unsigned k = counts[c];
        padded[c] = (k + 31u) & ~31u;
        atomicMax(maxc, k);
    }
}

// exact left-balanced k-d order inside one cell; writes the padded permutation
__global__ void __launch_bounds__(kCellThreads) k_cell_kd(const float4* __restrict__ a, const uint32_t* __restrict__ perm,
                                                          const unsigned* __restrict__ start,
                                                          const unsigned* __restrict__ count,
                                                          const unsigned* __restrict__ pstart, uint32_t* out) {
    extern __shared__ unsigned char smraw[];
    unsigned long long* key = (unsigned long long*)smraw;        // kCellMax
    float* X = (float*)(key + kCellMax);
    float* Y = X + kCellMax;
    float* Z = Y + kCellMax;
    uint32_t* ID = (uint32_t*)(Z + kCellMax);
    unsigned* blo = (unsigned*)(ID + kCellMax);                  // 3 * (kCellMax / 32)
    unsigned* bhi = blo + 3 * (kCellMax / 32);
    const uint32_t cell = blockIdx.x;
    const unsigned cnt = count[cell];
    if (cnt == 0) return;
    const unsigned P = (cnt + 31u) & ~31u;
    const unsigned Lc = P / 32;
    unsigned P2 = 32;
    while (P2 < P) P2 <<= 1;
    const unsigned s0 = start[cell];
    const float qnan = __int_as_float(0x7fc00000);
    for (unsigned j = threadIdx.x; j < P; j += blockDim.x) {
        if (j < cnt) {
            uint32_t id = perm[s0 + j];
            float4 p = a[id];
            X[j] = p.x; Y[j] = p.y; Z[j] = p.z; ID[j] = id;
        } else {
            X[j] = qnan; Y[j] = qnan; Z[j] = qnan; ID[j] = kDummy;
        }
    }
    __syncthreads();
    int depth = 0;
    while ((1u << depth) < Lc) ++depth;
    for (int d = 0; d < depth; ++d) {
        for (unsigned i = threadIdx.x; i < 3 * Lc; i += blockDim.x) {
            blo[i] = 0xffffffffu;
            bhi[i] = 0u;
        }
        __syncthreads();
        for (unsigned j = threadIdx.x; j < cnt; j += blockDim.x) {
            uint64_t na, nc;
            kd_node(j / 32, Lc, d, na, nc);
            if (nc > 1) {
                atomicMin(blo + 3 * na, f2ord(X[j])); atomicMax(bhi + 3 * na, f2ord(X[j]));
                atomicMin(blo + 3 * na + 1, f2ord(Y[j])); atomicMax(bhi + 3 * na + 1, f2ord(Y[j]));
                atomicMin(blo + 3 * na + 2, f2ord(Z[j])); atomicMax(bhi + 3 * na + 2, f2ord(Z[j]));
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
                    q = 0x1ffff;  // dummies sort last inside their node
                } else if (nc > 1) {
                    float l0 = ord2f(blo[3 * na]), l1 = ord2f(blo[3 * na + 1]), l2 = ord2f(blo[3 * na + 2]);
                    float e0 = ord2f(bhi[3 * na]) - l0, e1 = ord2f(bhi[3 * na + 1]) - l1, e2 = ord2f(bhi[3 * na + 2]) - l2;
                    float v, l, e;
                    if (e0 >= e1 && e0 >= e2) { v = X[j]; l = l0; e = e0; }
                    else if (e1 >= e2) { v = Y[j]; l = l1; e = e1; }
                    else { v = Z[j]; l = l2; e = e2; }
                    if (e > 0.f) q = (uint64_t)fminf(fmaxf((v - l) / e * 65535.f, 0.f), 65535.f);
                }
                k = (((na << 17) | q) << 13) | j;  // j < 8192 keeps equal keys in place
            }
            key[j] = k;
        }
        __syncthreads();
        // bitonic sort of P2 keys, ascending
        for (unsigned kk = 2; kk <= P2; kk <<= 1) {
            for (unsigned jj = kk >> 1; jj > 0; jj >>= 1) {
                for (unsigned i = threadIdx.x; i < P2; i += blockDim.x) {
                    unsigned p = i ^ jj;
                    if (p > i) {
                        unsigned long long x = key[i], y = key[p];
                        bool up = (i & kk) == 0;
                        if ((x > y) == up) {
                            key[i] = y;
                            key[p] = x;
                        }
                    }
                }
                __syncthreads();
            }
        }
        // gather the records into the new order (each thread keeps its own in registers)
        float rx[kCellMax / kCellThreads], ry[kCellMax / kCellThreads], rz[kCellMax / kCellThreads];
        uint32_t rid[kCellMax / kCellThreads];
        int t = 0;
        for (unsigned j = threadIdx.x; j < P; j += blockDim.x, ++t) {
            unsigned src = (unsigned)(key[j] & 0x1fffull);
            rx[t] = X[src]; ry[t] = Y[src]; rz[t] = Z[src]; rid[t] = ID[src];
        }
        __syncthreads();
        t = 0;
        for (unsigned j = threadIdx.x; j < P; j += blockDim.x, ++t) {
            X[j] = rx[t]; Y[j] = ry[t]; Z[j] = rz[t]; ID[j] = rid[t];
        }
        __syncthreads();
    }
    const unsigned o = pstart[cell];
    for (unsigned j = threadIdx.x; j < P; j += blockDim.x) out[o + j] = ID[j];
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

static size_t cell_smem_bytes() {
    return (size_t)kCellMax * 8 + (size_t)kCellMax * 16 + (size_t)2 * 3 * (kCellMax / 32) * 4;
}

// perm_out (capacity >= padded count) <- padded k-d order; returns the padded count or 0 on
// failure (cells too large after retries)
static uint64_t sampled_kd_order(Workspace& ws, const float4* a, uint64_t n, uint32_t* perm_out, uint64_t perm_cap,
                                 cudaStream_t st) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_cell_kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cell_smem_bytes());
        attr_set = true;
    }
    int T = 0;
    while ((n >> T) > (uint64_t)(kCellMax / 3)) ++T;
    for (int attempt = 0; attempt < 4; ++attempt, ++T) {
        size_t mark = ws.mark();
        const uint32_t ncell = 1u << T;
        uint8_t* axis = (uint8_t*)ws.take_bytes((uint64_t)ncell + 1);
        float* value = (float*)ws.take_bytes(((uint64_t)ncell + 1) * 4);
        if (T > 0) {
            uint64_t S = std::min<uint64_t>((uint64_t)ncell * 32, n);
            S = 1ull << (63 - __builtin_clzll(S));  // power of two
            if (S < ((uint64_t)ncell << 1)) S = (uint64_t)ncell << 1;
            uint64_t stride = std::max<uint64_t>(n / S, 1);
            float4* smp = (float4*)ws.take_bytes(S * 16);
            float4* smp2 = (float4*)ws.take_bytes(S * 16);
            uint32_t* sp = ws.take_u32(S);
            uint32_t* sp2 = ws.take_u32(S);
            unsigned blocks = (unsigned)std::min<uint64_t>((S + 255) / 256, 8192);
            k_take_sample<<<blocks, 256, 0, st>>>(a, n, stride, S, smp);
            note_launch();
            // k-d order of the sample with the level-synchronous builder: 32-record
            // leaves, so levels above 5 split the sample in power-of-two halves
            kd_order(ws, smp, S, sp, sp2, st);
            k_permute4<<<blocks, 256, 0, st>>>(smp, sp, smp2, S);
            note_launch();
            k_top_planes<<<ncell - 1, 256, 0, st>>>(smp2, S, axis, value);
            note_launch();
        }
        unsigned* counts = ws.take_u32(ncell);
        unsigned* padded = ws.take_u32(ncell);
        unsigned* starts = ws.take_u32(ncell);
        unsigned* pstarts = ws.take_u32(ncell);
        uint64_t* keys = (uint64_t*)ws.take_bytes(n * 8);
        uint64_t* keys2 = (uint64_t*)ws.take_bytes(n * 8);
        uint32_t* vals = ws.take_u32(n);
        uint32_t* vals2 = ws.take_u32(n);
        unsigned* maxc = ws.scratch_box();
        cudaMemsetAsync(counts, 0, (size_t)ncell * 4, st);
        cudaMemsetAsync(maxc, 0, 4, st);
        unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 16384);
        k_assign_cells<<<blocks, 256, 0, st>>>(a, n, T, axis, value, keys, vals, counts);
        note_launch();
        k_pad_counts<<<(ncell + 255) / 256, 256, 0, st>>>(counts, ncell, padded, maxc);
        note_launch();
        unsigned hmax = 0;
        cudaMemcpyAsync(&hmax, maxc, 4, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        if (hmax > (unsigned)kCellMax) {  // unlucky sample: more cells
            ws.release(mark);
            continue;
        }
        cudaMemcpyAsync(starts, counts, (size_t)ncell * 4, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(pstarts, padded, (size_t)ncell * 4, cudaMemcpyDeviceToDevice, st);
        exclusive_scan(ws, starts, ncell, st);
        exclusive_scan(ws, pstarts, ncell, st);
        unsigned last_ps = 0, last_pad = 0;
        cudaMemcpyAsync(&last_ps, pstarts + ncell - 1, 4, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&last_pad, padded + ncell - 1, 4, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        uint64_t total = (uint64_t)last_ps + last_pad;
        if (total > perm_cap) {
            ws.release(mark);
            return 0;
        }
        if (T > 0) radix_sort_pairs(ws, keys, vals, keys2, vals2, n, (uint64_t)ncell - 1, st);
        k_cell_kd<<<ncell, kCellThreads, cell_smem_bytes(), st>>>(a, vals, starts, counts, pstarts, perm_out);
        note_launch();
        ws.release(mark);
        return total;
    }
    return 0;
}

// ------------------------------------------------------------------------------------------
// permutation and box tree
// ------------------------------------------------------------------------------------------

__global__ void k_permute4(const float4* __restrict__ src, const uint32_t* __restrict__ perm,
                           float4* __restrict__ dst, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

__global__ void k_permute_u32(const uint32_t* __restrict__ src, const uint32_t* __restrict__ perm,
                              uint32_t* __restrict__ dst, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

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

KeyGrid make_key_grid(const float lo[3], const float hi[3]) {
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
    int bits = na == 3 ? 21 : 32;  // 63-bit keys in 3-D, 64-bit for planar maps
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

int compute_bbox(Workspace& ws, const float4* a, uint64_t n, float lo[3], float hi[3], cudaStream_t st) {
    unsigned* box = ws.scratch_box();
    unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    cudaMemcpyAsync(box, init, sizeof(init), cudaMemcpyHostToDevice, st);
    unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 4096);
    if (blocks == 0) blocks = 1;
    k_bbox<<<blocks, 256, 0, st>>>(a, nullptr, n, box);
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

// Sort the records of one channel into Morton order and build the box tree.
int build_map_index(Workspace& ws, const RecordStore& rec, uint64_t n, MapIndex& m, cudaStream_t st) {
    m.n = n;
    m.n_real = n;
    if (n == 0) {
        m.nlevels = 0;
        return 0;
    }
    float lo[3], hi[3];
    compute_bbox(ws, rec.a, n, lo, hi, st);
    m.grid = make_key_grid(lo, hi);
    size_t mark = ws.mark();
    uint32_t* vals = ws.take_u32(n);
    uint32_t* vals2 = ws.take_u32(n);
    kd_order(ws, rec.a, n, vals, vals2, st);
    const uint64_t np = n;
    m.n_real = n;
    m.n = np;
    unsigned blocks = (unsigned)std::min<uint64_t>((np + 255) / 256, 8192);
    m.a = (float4*)ws.alloc_persistent(m.a, m.a_cap, np);
    m.b = (float4*)ws.alloc_persistent(m.b, m.b_cap, np);
    k_permute4_pad<<<blocks, 256, 0, st>>>(rec.a, vals, m.a, np);
    note_launch();
    k_permute4_pad<<<blocks, 256, 0, st>>>(rec.b, vals, m.b, np);
    note_launch();
    if (rec.fwi) {
        m.fwi = (float4*)ws.alloc_persistent(m.fwi, m.fwi_cap, np);
        m.sfi = (float4*)ws.alloc_persistent(m.sfi, m.sfi_cap, np);
        k_permute4_pad<<<blocks, 256, 0, st>>>(rec.fwi, vals, m.fwi, np);
        note_launch();
        k_permute4_pad<<<blocks, 256, 0, st>>>(rec.sfi, vals, m.sfi, np);
        note_launch();
    }
    if (rec.id) {
        m.id = (uint32_t*)ws.alloc_persistent_u32(m.id, m.id_cap, np);
        k_permute_u32_pad<<<blocks, 256, 0, st>>>(rec.id, vals, m.id, np);
        note_launch();
    }
    build_box_tree(ws, m, st);
    ws.release(mark);
    return 0;
}

// Single-cell index build into caller-provided device memory (no allocation): the k-d
// order of n <= kCellMax points (one CTA), the padded permuted copy and its box tree.
// `cell` holds {start = 0, count = n, pstart = 0}; perm_in is the identity.
int cell_index_max_points() { return kCellMax; }

void launch_single_cell_index(const float4* pts, uint32_t n, const uint32_t* perm_in, const unsigned* cell,
                              uint32_t* perm_out, float4* sorted, float4* box_lo, float4* box_hi,
                              const uint64_t* lvl_off, const uint64_t* lvl_cnt, int nlevels, cudaStream_t st) {
    static bool attr_set[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        cudaFuncSetAttribute(k_cell_kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cell_smem_bytes());
        attr_set[dev] = true;
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
int sort_queries(Workspace& ws, const float4* qa, uint64_t n, const KeyGrid& g, uint32_t* perm,
                 cudaStream_t st) {
    if (n == 0) return 0;
    size_t mark = ws.mark();
    uint64_t* keys = (uint64_t*)ws.take_bytes(n * 8);
    uint32_t* vals = perm;
    uint64_t* keys2 = (uint64_t*)ws.take_bytes(n * 8);
    uint32_t* vals2 = ws.take_u32(n);
    unsigned long long* oa = (unsigned long long*)ws.scratch_box();
    unsigned long long init[2] = {0ull, ~0ull};
    cudaMemcpyAsync(oa, init, sizeof(init), cudaMemcpyHostToDevice, st);
    unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 8192);
    k_keys<<<blocks, 256, 0, st>>>(qa, n, g, keys, vals, oa);
    note_launch();
    unsigned long long h[2];
    cudaMemcpyAsync(h, oa, sizeof(h), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    uint64_t* k0 = keys;
    uint32_t* v0 = vals;
    radix_sort_pairs(ws, k0, v0, keys2, vals2, n, h[0] ^ h[1], st);
    if (v0 != perm) cudaMemcpyAsync(perm, v0, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    ws.release(mark);
    return 0;
}

}  // namespace alb
