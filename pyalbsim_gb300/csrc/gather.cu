// Photon-map gather: exact k-nearest-neighbour density estimation at every backward event
// and time-binned waveform accumulation. GPU form of Simulation.sample_photons
// (alb_sim/core/simulation.py:132-214) with scipy KDTree.query(x, k) as the neighbour
// search (alb_sim/photon_mapping/photon_map_index.py:17).
//
// One warp per query. The warp walks the 32-ary box tree depth first, nearest child
// first (children sorted by box distance with a warp bitonic sort), keeps candidates in a
// shared-memory buffer and shrinks it to the k best with a warp radix select whenever it
// fills. Distances are float32 for the search; the threshold carries a relative margin
// of 2^-18 so that every point whose float64 distance could rank at the k-th place
// survives, and the boundary band is resolved with float64 distances exactly as the
// reference's KDTree (float64 on float32-cast map positions) orders them.
//
// Each warp takes contiguous chunks of the spatially sorted queries; from the second query
// of a chunk on, the search starts with the largest distance from the query to the previous
// query's k neighbours (k points lie within it, so it bounds the k-th distance; never looser
// than the triangle bound r_k(prev) + |q - prev|), inflated by 2^-14 so that every point of
// the float32 boundary band is still admitted.
#include <cfloat>

#include "device_common.cuh"
#include "internal.h"

namespace alb {

constexpr int kGatherWarps = 8;   // 8-warp CTAs, 4 per SM: 32 warps hide the gather's latency
constexpr int kGatherBlocksPerSM = 4;
// consecutive sorted queries handled by one warp: each chunk's first search runs without a
// bound, longer chunks balance worse (scatter map at 1e7 photons: 32 -> 546 ms, 64 -> 529 ms,
// 128 -> 524 ms; the planar maps' gathers lose 2-3% at 128)
constexpr int kQueryChunk = 64;
constexpr int kQueryChunkScatter = 128;
constexpr int kStack = 32 * kMaxLevels;
constexpr int kCap = 288;         // candidate buffer (k <= kCap - 32)
constexpr int kSelectAt = 192;    // shrink the buffer once it holds more than this
constexpr int kBand = 32;         // near-tie entries resolved in float64
constexpr int kLeafList = 2 * kBand;  // leaf list of a search under a guess (aliases the band)
// Squared widening of the previous query's k-th distance that the scatter-map search first
// admits within (1.1^2): consecutive sorted queries' k-th distances differ by less than 10%
// for 97% of them; a guess that does not hold is detected and the search redone (measured
// at 1e7 photons: 1.1^2 gave the fastest scatter gather of 1.1^2, 1.15^2 and 1.2^2).
constexpr float kGuessWiden2 = 1.21f;
// Admission margin of the float32 screening distance (its error is below 2^-22 relative).
constexpr float kRelMargin = 9.5367431640625e-07f;  // 2^-20

// Candidates carry an error-free double-float squared distance, stored as its float32 high
// part cd and a 16-bit fraction cl of one ulp of cd (key48 = cd bits : cl + 2^15 orders
// them to ~2^-40 relative); only entries within one key unit of the k-th are resolved in
// float64.
struct WarpSmem {
    uint32_t stk[kStack];
    float stk_d[kStack];
    float cd[kCap];
    uint32_t ci[kCap];
    int16_t cl[kCap];
    uint32_t hist[128];  // 256 radix bins, two 16-bit counters per word
    union {
        double bd[kBand];               // near-tie band: float64 distances (after the search)
        uint32_t leafl[kLeafList];      // leaves to screen (during a search under a guess)
    };
    uint32_t bi[kBand];  // map positions
    uint64_t bt[kBand];  // tie keys from the record's content (or 0)
    float prev_rk2;      // squared k-th distance of the warp's previous query (kept out of registers)
    unsigned long long st[5];  // the warp's search counters: leaves, nodes, selects, queries, inexact
};

// Lower bound of the squared distance from the float64 query (qx + lx, ...) to a box:
// the float32 per-axis gap is shrunk by its rounding bound and by the dropped low part,
// so that pruning never discards a box the float64 search would have to open.
ALB_DEVICE float box_gap(float lo, float hi, float q, float ql) {
    float g = fmaxf(fmaxf(lo - q, q - hi), 0.f);
    return fmaxf(g * (1.f - 2.384185791015625e-07f) - fabsf(ql), 0.f);
}
ALB_DEVICE float box_dist2(float qx, float qy, float qz, float lx, float ly, float lz, float4 lo, float4 hi) {
    float dx = box_gap(lo.x, hi.x, qx, lx);
    float dy = box_gap(lo.y, hi.y, qy, ly);
    float dz = box_gap(lo.z, hi.z, qz, lz);
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * (1.f - 4.76837158203125e-07f);
}

// float32 distance of a map point to the query (hi + lo split of the float64 position)
ALB_DEVICE float point_dist2(float qx, float qy, float qz, float lx, float ly, float lz, float4 p) {
    float dx = (p.x - qx) - lx;
    float dy = (p.y - qy) - ly;
    float dz = (p.z - qz) - lz;
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

ALB_DEVICE double point_dist2_f64(double qx, double qy, double qz, float4 p) {
    double dx = (double)p.x - qx, dy = (double)p.y - qy, dz = (double)p.z - qz;
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Error-free transforms (Knuth two-sum); the _rn intrinsics keep the compiler from fusing
// the operations into FMAs, which would break the error terms.
ALB_DEVICE void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Squared distance from the query (f + l per axis) to p as hi + lo with about 2^-44
// relative error: exact per-axis differences by two-sum, squares by FMA two-product.
ALB_DEVICE void point_dist2_df(float fx, float fy, float fz, float lx, float ly, float lz, float4 p, float& hi,
                               float& lo) {
    float sx, ex, sy, ey, sz, ez;
    two_sum(p.x, -fx, sx, ex);
    two_sum(p.y, -fy, sy, ey);
    two_sum(p.z, -fz, sz, ez);
    float hx, tx, hy, ty, hz, tz;
    two_sum(sx, __fsub_rn(ex, lx), hx, tx);
    two_sum(sy, __fsub_rn(ey, ly), hy, ty);
    two_sum(sz, __fsub_rn(ez, lz), hz, tz);
    const float px = __fmul_rn(hx, hx), py = __fmul_rn(hy, hy), pz = __fmul_rn(hz, hz);
    const float qx = fmaf(2.f * hx, tx, fmaf(hx, hx, -px));
    const float qy = fmaf(2.f * hy, ty, fmaf(hy, hy, -py));
    const float qz = fmaf(2.f * hz, tz, fmaf(hz, hz, -pz));
    float s1, e1, s2, e2;
    two_sum(px, py, s1, e1);
    two_sum(s1, pz, s2, e2);
    const float t = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fadd_rn(qx, qy), qz));
    hi = __fadd_rn(__fadd_rn(s2, t), 0.f);  // (+0 for an exact zero)
    lo = __fsub_rn(t, __fsub_rn(hi, s2));
}

// lo in units of 2^-16 ulp(hi), clamped to 16 bits
ALB_DEVICE int16_t frac16(float hi, float lo) {
    const int e = (int)((__float_as_uint(hi) >> 23) & 255u);
    if (e == 0) return 0;
    const int sh = min(166 - e, 127);  // 2^(16 + 23 - (e - 127))
    float q = lo * __uint_as_float((uint32_t)(sh + 127) << 23);
    q = fminf(fmaxf(rintf(q), -32767.f), 32767.f);
    return (int16_t)q;
}

ALB_DEVICE uint64_t cand_key(const WarpSmem& s, int i) {
    return ((uint64_t)__float_as_uint(s.cd[i]) << 16) | (uint32_t)((int)s.cl[i] + 32768);
}

// float32(sqrt(x)) for a double x >= 0, correctly rounded (equal to casting the float64
// square root, as double rounding is harmless for sqrt from 53 to 24 bits): a float32
// estimate corrected against the squared float midpoints, which are exact in float64.
ALB_DEVICE float sqrt_to_f32(double x) {
    if (!(x > 0.0)) return 0.f;
    float s = sqrtf(__double2float_rn(x));
    const float up = __int_as_float(__float_as_int(s) + 1);
    const float dn = __int_as_float(__float_as_int(s) - 1);
    const double mh = 0.5 * ((double)s + (double)up), ml = 0.5 * ((double)s + (double)dn);
    const double mh2 = mh * mh, ml2 = ml * ml;
    if (x > mh2 || (x == mh2 && (__float_as_int(up) & 1) == 0)) s = up;
    else if (x < ml2 || (x == ml2 && (__float_as_int(dn) & 1) == 0)) s = dn;
    return s;
}

// Tie key of a map record: its time bits (high word; times are non-negative) and a 32-bit
// mix of its direction, time and energy bits (low word).
ALB_DEVICE uint64_t record_tie_key(float4 a, float4 b) {
    uint32_t h = 0x9e3779b9u;
    const uint32_t w[4] = {__float_as_uint(b.x), __float_as_uint(b.y), __float_as_uint(b.z), __float_as_uint(a.w)};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        h ^= w[i] * 0x85ebca6bu;
        h = (h << 13) | (h >> 19);
        h = h * 5u + 0xe6546b64u;
    }
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    return ((uint64_t)__float_as_uint(b.w) << 32) | h;
}

// Warp bitonic sort of 32 (key, value) pairs, ascending by key. The stages are a loop, not
// an unrolled network: the gather is bound by instruction fetch, and the rolled form keeps
// its hot code smaller (measured 12% faster for the scatter-map gather).
ALB_DEVICE void warp_sort32(float& key, uint32_t& val) {
    const int l = lane_id();
#pragma unroll 1
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll 1
        for (int j = k >> 1; j > 0; j >>= 1) {
            float ok = __shfl_xor_sync(0xffffffffu, key, j);
            uint32_t ov = __shfl_xor_sync(0xffffffffu, val, j);
            bool up = ((l & k) == 0);
            bool lower = ((l & j) == 0);
            bool take_other = lower ? (up ? ok < key : ok > key) : (up ? ok > key : ok < key);
            if (take_other) {
                key = ok;
                val = ov;
            }
        }
    }
}

// Shared radix-select step: from the 256-bin histogram in s.hist (two 16-bit counters per
// word) pick the digit holding the need-th (1-based) entry; need becomes its rank inside.
ALB_DEVICE uint32_t radix_pick(const WarpSmem& s, int& need) {
    const int l = lane_id();
    uint32_t h[8], run = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t w = s.hist[l * 4 + j];
        h[2 * j] = w & 0xffffu;
        h[2 * j + 1] = w >> 16;
        run += h[2 * j] + h[2 * j + 1];
    }
    uint32_t incl = run;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (l >= o) incl += t;
    }
    uint32_t before = incl - run;
    int digit = -1;
    uint32_t below = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (digit < 0 && before + h[j] >= (uint32_t)need) {
            digit = l * 8 + j;
            below = before;
        }
        before += h[j];
    }
    const unsigned who = __ballot_sync(0xffffffffu, digit >= 0);
    const int src = __ffs(who) - 1;
    digit = __shfl_sync(0xffffffffu, digit, src);
    below = __shfl_sync(0xffffffffu, below, src);
    need -= (int)below;
    return (uint32_t)digit;
}

// k-th smallest (1-based) float32 part cd[off .. off + cnt) (all >= 0): warp radix select.
ALB_DEVICE float warp_kth32(WarpSmem& s, int off, int cnt, int k) {
    const int l = lane_id();
    uint32_t prefix = 0u, pmask = 0u;
    int need = k;
#pragma unroll 1
    for (int shift = 24; shift >= 0; shift -= 8) {
#pragma unroll 1
        for (int i = l; i < 128; i += 32) s.hist[i] = 0u;
        __syncwarp();
#pragma unroll 1
        for (int i = l; i < cnt; i += 32) {
            const uint32_t u = __float_as_uint(s.cd[off + i]);
            if ((u & pmask) == prefix) {
                const uint32_t d = (u >> shift) & 255u;
                atomicAdd(&s.hist[d >> 1], 1u << ((d & 1u) * 16u));
            }
        }
        __syncwarp();
        prefix |= radix_pick(s, need) << shift;
        pmask |= 255u << shift;
        __syncwarp();
    }
    return __uint_as_float(prefix);
}

// k-th smallest (1-based) float32 part cd[0 .. cnt), for candidates that mostly lie in
// [0, hi]: one pass of 256 linear bins over [0, hi] (bin = d * 256 / hi, truncated and
// clamped, which is monotone in d, so the bins keep the order), then an exact rank among the
// entries of the bin that holds the k-th (usually one to three). Falls back to the four-pass
// radix select when hi gives no spread or that bin holds more than 32 entries.
ALB_DEVICE float warp_kth32_lin(WarpSmem& s, int cnt, int k, float hi) {
    const float scale = 256.f / hi;
    if (!(hi > 0.f) || !(scale < 1.0e30f)) return warp_kth32(s, 0, cnt, k);
    const int l = lane_id();
#pragma unroll 1
    for (int i = l; i < 128; i += 32) s.hist[i] = 0u;
    __syncwarp();
#pragma unroll 1
    for (int i = l; i < cnt; i += 32) {
        const uint32_t d = (uint32_t)min((int)(s.cd[i] * scale), 255);
        atomicAdd(&s.hist[d >> 1], 1u << ((d & 1u) * 16u));
    }
    __syncwarp();
    int need = k;
    const uint32_t B = radix_pick(s, need);  // need: rank inside bin B (1-based)
    __syncwarp();
    int m = 0;
#pragma unroll 1
    for (int base = 0; base < cnt; base += 32) {
        const int i = base + l;
        const float d = i < cnt ? s.cd[i] : 0.f;
        const bool in = i < cnt && (uint32_t)min((int)(d * scale), 255) == B;
        const unsigned b = __ballot_sync(0xffffffffu, in);
        if (in) {
            const int pos = m + __popc(b & lanemask_lt());
            if (pos < 32) s.hist[pos] = __float_as_uint(d);
        }
        m += __popc(b);
    }
    __syncwarp();
    if (m > 32) return warp_kth32(s, 0, cnt, k);
    const float v = l < m ? __uint_as_float(s.hist[l]) : FLT_MAX;
    int rank = 0;
#pragma unroll 1
    for (int j = 0; j < m; ++j) {
        const float o = __shfl_sync(0xffffffffu, v, j);
        rank += (o < v || (o == v && j < l)) ? 1 : 0;
    }
    const unsigned own = __ballot_sync(0xffffffffu, l < m && rank == need - 1);
    const float kth = __shfl_sync(0xffffffffu, v, __ffs(own) - 1);
    __syncwarp();
    return kth;
}

// k-th smallest (1-based) 48-bit candidate key by warp radix select over its top
// 8 * PASSES bits (PASSES = 4: the float32 part only; the lower bits return as 0).
template <int PASSES>
ALB_DEVICE uint64_t warp_kth_key(WarpSmem& s, int off, int cnt, int k) {
    const int l = lane_id();
    uint64_t prefix = 0ull, pmask = 0ull;
    int need = k;
#pragma unroll 1
    for (int pass = 0; pass < PASSES; ++pass) {
        const int shift = 40 - 8 * pass;
        for (int i = l; i < 128; i += 32) s.hist[i] = 0u;
        __syncwarp();
        for (int i = l; i < cnt; i += 32) {
            const uint64_t u = cand_key(s, off + i);
            if ((u & pmask) == prefix) {
                const uint32_t d = (uint32_t)(u >> shift) & 255u;
                atomicAdd(&s.hist[d >> 1], 1u << ((d & 1u) * 16u));
            }
        }
        __syncwarp();
        prefix |= ((uint64_t)radix_pick(s, need)) << shift;
        pmask |= 255ull << shift;
        __syncwarp();
    }
    return prefix;
}

// Keep the candidates whose float32 part is <= thr (order not preserved).
ALB_DEVICE int warp_compact(WarpSmem& s, int cnt, float thr) {
    const int l = lane_id();
    int out = 0;
#pragma unroll 1
    for (int base = 0; base < cnt; base += 32) {
        int i = base + l;
        float d = i < cnt ? s.cd[i] : FLT_MAX;
        uint32_t id = i < cnt ? s.ci[i] : 0u;
        int16_t lo = i < cnt ? s.cl[i] : (int16_t)0;
        bool keep = i < cnt && d <= thr;
        unsigned b = __ballot_sync(0xffffffffu, keep);
        __syncwarp();
        if (keep) {
            int pos = out + __popc(b & lanemask_lt());
            s.cd[pos] = d;
            s.ci[pos] = id;
            s.cl[pos] = lo;
        }
        out += __popc(b);
        __syncwarp();
    }
    return out;
}


struct KnnResult {
    double rk2;    // float64 squared distance of the k-th neighbour
    float rkf;     // float32(sqrt(rk2)), correctly rounded
    int leaves;    // leaves opened (32 records each)
    int nodes;     // internal nodes expanded
    int selects;   // candidate-buffer reductions
    int clipped;   // 1 if a buffer bound forced an inexact answer (mass ties)
    int retried;   // 1 if an optimistic first threshold did not hold and the search was redone
    int fail;      // 0, or why the search has no answer (s.ci is then not valid):
                   // ALB_ERR_ITER_CAP (traversal guard) or ALB_ERR_INVALID (fewer than k
                   // finite points admitted: a NaN or infinite query or map coordinates)
};

// float64 ranking of the band entries bi[0..nb) by (distance, tie key, map position); the
// `take` smallest go to ci[dst ..] in rank order. Returns the float64 squared distance of
// the take-th (0 if the band holds fewer).
ALB_DEVICE double rank_band(const MapDev& m, WarpSmem& s, int dst, int nb, int take, double qx, double qy,
                            double qz, const float4* tie_rec) {
    const int l = lane_id();
    double di = 0.0;
    uint64_t ti = 0ull;
    uint32_t ii = 0u;
    int rank = 0;
    if (l < nb) {
        ii = s.bi[l];
        const float4 a = m.a[ii];
        di = point_dist2_f64(qx, qy, qz, a);
        ti = tie_rec ? record_tie_key(a, tie_rec[ii]) : 0ull;
        s.bd[l] = di;
        s.bt[l] = ti;
    }
    __syncwarp();
    if (l < nb) {
#pragma unroll 1
        for (int j = 0; j < nb; ++j) {
            const double dj = s.bd[j];
            const uint64_t tj = s.bt[j];
            rank += (dj < di || (dj == di && (tj < ti || (tj == ti && s.bi[j] < ii)))) ? 1 : 0;
        }
    }
    __syncwarp();
    if (l < nb && rank < take) s.ci[dst + rank] = ii;
    const unsigned owner = __ballot_sync(0xffffffffu, l < nb && rank == take - 1);
    const double rk2 = owner ? __shfl_sync(0xffffffffu, di, __ffs(owner) - 1) : 0.0;
    __syncwarp();
    return rk2;
}

// The k_sub nearest among the entries [off, off + n) whose cd/cl hold refined keys: keys more
// than one unit below the k_sub-th are in, keys within one unit of it are ranked in float64.
// The chosen map positions end up in ci[off .. off + k_sub).
ALB_DEVICE double select_refined(const MapDev& m, WarpSmem& s, int off, int n, int k_sub, double qx, double qy,
                                 double qz, const float4* tie_rec, int& clipped) {
    const int l = lane_id();
    const uint64_t K = warp_kth_key<6>(s, off, n, k_sub);
    int n_in = 0, n_band = 0;
#pragma unroll 1
    for (int base = 0; base < n; base += 32) {
        const bool valid = base + l < n;
        const int i = off + base + l;
        const uint64_t key = valid ? cand_key(s, i) : ~0ull;
        const uint32_t id = valid ? s.ci[i] : 0u;
        const bool in = valid && key + 1ull < K;
        const bool band = valid && !in && key <= K + 1ull;
        const unsigned bin = __ballot_sync(0xffffffffu, in);
        const unsigned bb = __ballot_sync(0xffffffffu, band);
        __syncwarp();
        if (in) s.ci[off + n_in + __popc(bin & lanemask_lt())] = id;
        if (band) {
            const int pos = n_band + __popc(bb & lanemask_lt());
            if (pos < kBand) s.bi[pos] = id;
        }
        n_in += __popc(bin);
        n_band += __popc(bb);
        __syncwarp();
    }
    if (n_band > kBand) {
        n_band = kBand;
        clipped = 1;
    }
    return rank_band(m, s, off + n_in, n_band, k_sub - n_in, qx, qy, qz, tie_rec);
}

// Full k-NN search for one query. Returns false when the map has fewer than k records; the
// k nearest map positions are then in s.ci[0 .. k).
// thr_safe: an upper bound of the squared k-th distance that already includes the band margin
// (FLT_MAX when none is known). thr0 <= thr_safe: the first search's threshold, which may be
// an optimistic guess. A search under a guess is accepted only when its own answer proves it
// complete: at least k candidates, and the k-th with its band margin within the guess (every
// point that can rank among the k nearest then had a distance below the admission
// threshold, and every box holding one was opened). Otherwise the search is repeated under
// thr_safe, and under no bound at all if that fails too. Either way the answer is the one a
// search from no bound gives.
// The query is (fx + lx, fy + ly, fz + lz) = (qx, qy, qz) exactly, |l*| <= half an ulp of f*.
// Points at exactly the same float64 distance rank by a key taken from their record content
// (time, then a hash of direction, time and energy; when tie_rec is given) and then by map
// position, so that the chosen neighbours do not depend on the order in which the map's
// records are stored (records equal in all of these contribute identically).
// REFINE: candidates carry double-float distances from admission on, so the buffer only ever
// holds entries within one float32 ulp of the k-th: needed where many points sit at nearly
// the same distance (queries far from a dense planar map). Without it candidates carry the
// float32 screening distance and only a crowded final band is refined.
template <bool REFINE, bool QSPLIT = false>
ALB_DEVICE bool warp_knn(const MapDev& m, WarpSmem& s, int k, double qx, double qy, double qz, float fx,
                         float fy, float fz, float lx, float ly, float lz, float thr0, float thr_safe,
                         const float4* tie_rec, KnnResult& res) {
    const int l = lane_id();
    if (m.n_real < (uint64_t)k) return false;
    float thr = thr0;  // admission threshold (float32 squared distance, with margin)
    int cnt = 0;
    float kth_known = -1.f;  // the float32 k-th of the accepted search (!REFINE), when computed
    res.leaves = res.nodes = res.selects = res.clipped = res.retried = res.fail = 0;
    // Thresholds in turn: the first guess, the safe bound, no bound. A carried safe bound can
    // only fail through a degenerate previous result (a clipped boundary band).
    float start = thr0;
    for (int attempt = 0; attempt < 3; ++attempt) {
        if (attempt == 1) {
            if (!(thr_safe > thr0)) continue;  // the guess was the safe bound itself
            start = thr_safe;
            res.retried = 1;
        }
        if (attempt == 2) {
            if (start == FLT_MAX) break;
            start = FLT_MAX;
        }
        thr = start;
        cnt = 0;
        int sp = 0;
        // roots
        {
            int top = m.nlevels - 1;
            uint64_t ntop = m.lvl_cnt[top];
            float d = FLT_MAX;
            uint32_t c = (uint32_t)l;
            if ((uint64_t)l < ntop) {
                d = box_dist2(fx, fy, fz, lx, ly, lz, m.box_lo[m.lvl_off[top] + l], m.box_hi[m.lvl_off[top] + l]);
                if (d > thr) d = FLT_MAX;
            }
            warp_sort32(d, c);
            unsigned b = __ballot_sync(0xffffffffu, d < FLT_MAX);
            int nv = __popc(b);
            if (l < nv) {
                s.stk[sp + nv - 1 - l] = ((uint32_t)top << 29) | c;
                s.stk_d[sp + nv - 1 - l] = d;
            }
            sp += nv;
            __syncwarp();
        }
        int guard = 0;
        // Under a guessed threshold the threshold rarely shrinks, so the order of the boxes
        // does not change which leaves are opened: the leaves of expanded leaf parents are
        // collected in s.leafl and screened in batches, with the next leaf's records loaded
        // while the current leaf is screened, so the leaf visits do not form one chain of
        // dependent loads. The ordered search (a safe bound, or none) takes its leaves from
        // the stack, nearest first.
        const bool listed = !REFINE && start < thr_safe;
        int nlist = 0;
        // screen the 32 records of leaf `leaf` (p = this lane's record) against the threshold
        auto admit = [&](uint32_t leaf, float4 p) {
            ++res.leaves;
            const uint64_t r = (uint64_t)leaf * 32 + l;
            const bool real = r < m.n;  // the last leaf may be partial
            const float d = real ? point_dist2(fx, fy, fz, lx, ly, lz, p) : FLT_MAX;
            const bool take = real && d <= thr;
            const unsigned b = __ballot_sync(0xffffffffu, take);
            if (take) {
                const int pos = cnt + __popc(b & lanemask_lt());
                s.ci[pos] = (uint32_t)r;
                if (REFINE) {
                    float hi, lo;
                    point_dist2_df(fx, fy, fz, lx, ly, lz, p, hi, lo);
                    s.cd[pos] = hi;
                    s.cl[pos] = frac16(hi, lo);
                } else {
                    s.cd[pos] = d;
                }
            }
            cnt += __popc(b);
            __syncwarp();
            if (cnt >= k && (thr == FLT_MAX || cnt > kSelectAt)) {
                ++res.selects;
                // planar maps (REFINE) crowd their candidates into one linear bin: radix select
                const float kth = REFINE ? warp_kth32(s, 0, cnt, k) : warp_kth32_lin(s, cnt, k, thr);
                thr = fminf(thr, kth * (1.0f + 2.0f * kRelMargin));
                // REFINE: refined distances within one float32 ulp of the k-th can still
                // rank among the k nearest, nothing beyond can; otherwise the float32
                // screening margin decides
                cnt = warp_compact(s, cnt, REFINE ? __uint_as_float(__float_as_uint(kth) + 1u) : thr);
                if (cnt > kCap - 32) {  // mass ties
                    cnt = warp_compact(s, cnt, kth);
                    res.clipped = 1;
                }
                if (cnt > kCap - 32) cnt = kCap - 32;  // keeps the buffer in bounds
            }
        };
        auto load_leaf = [&](uint32_t leaf) {
            const uint64_t r = (uint64_t)leaf * 32 + l;
            return r < m.n ? m.a[r] : make_float4(0.f, 0.f, 0.f, 0.f);
        };
        auto flush = [&]() {
#pragma unroll 1
            for (int i = 0; i < nlist; ++i) admit(s.leafl[i], load_leaf(s.leafl[i]));
            nlist = 0;
        };
        while (sp > 0) {
            if (++guard > (1 << 22)) {  // reported, never a silent partial answer
                res.fail = ALB_ERR_ITER_CAP;
                break;
            }
            uint32_t etop;
            {
                // the top 32 stack entries, one per lane (lane 0 = top)
                const int i = sp - 1 - l;
                uint32_t e = 0u;
                bool ok = false;
                if (i >= 0) {
                    e = s.stk[i];
                    ok = s.stk_d[i] <= thr;
                }
                const unsigned okm = __ballot_sync(0xffffffffu, ok);
                if (!okm) {  // 32 entries beyond the threshold
                    sp = sp > 32 ? sp - 32 : 0;
                    __syncwarp();
                    continue;
                }
                const int f = __ffs(okm) - 1;
                etop = __shfl_sync(0xffffffffu, e, f);
                sp -= f + 1;
                __syncwarp();
            }
            if ((etop >> 29) == 0) {
                // a leaf of the ordered search: admit its points within the threshold
                admit(etop, load_leaf(etop));
            } else {
                ++res.nodes;
                const int lev = (int)(etop >> 29);
                const uint32_t node = etop & 0x1fffffffu;
                uint64_t c = (uint64_t)node * 32 + l;
                float d = FLT_MAX;
                int cl = lev - 1;
                if (c < m.lvl_cnt[cl]) {
                    d = box_dist2(fx, fy, fz, lx, ly, lz, m.box_lo[m.lvl_off[cl] + c], m.box_hi[m.lvl_off[cl] + c]);
                    if (d > thr) d = FLT_MAX;
                }
                uint32_t cc = (uint32_t)c;
                const unsigned vm = __ballot_sync(0xffffffffu, d < FLT_MAX);
                int nv = __popc(vm);
                if (listed) {
                    // children are taken as they come, without ordering them; leaves go to
                    // the list
                    if (d < FLT_MAX) {
                        const int pos = __popc(vm & lanemask_lt());
                        if (cl == 0) {
                            s.leafl[nlist + pos] = cc;
                        } else {
                            s.stk[sp + pos] = ((uint32_t)cl << 29) | cc;
                            s.stk_d[sp + pos] = d;
                        }
                    }
                    if (cl == 0) {
                        nlist += nv;
                        nv = 0;
                    }
                } else if (nv <= 16) {
                    // few children within the threshold: extract them nearest first
                    // (non-negative floats order like their bit patterns)
                    unsigned key = __float_as_uint(d);
                    for (int r = 0; r < nv; ++r) {
                        unsigned mn = __reduce_min_sync(0xffffffffu, key);
                        int src = __ffs(__ballot_sync(0xffffffffu, key == mn)) - 1;
                        if (l == src) {
                            s.stk[sp + nv - 1 - r] = ((uint32_t)cl << 29) | cc;
                            s.stk_d[sp + nv - 1 - r] = d;
                            key = 0xffffffffu;
                        }
                    }
                } else {
                    warp_sort32(d, cc);
                    if (l < nv) {
                        s.stk[sp + nv - 1 - l] = ((uint32_t)cl << 29) | cc;
                        s.stk_d[sp + nv - 1 - l] = d;
                    }
                }
                sp += nv;
                __syncwarp();
                if (nlist > kLeafList - 32) flush();  // room for the next parent's 32 leaves
            }
        }
        if (!res.fail) flush();
        if (res.fail || start == FLT_MAX) break;
        if (cnt < k) continue;
        if (REFINE || start >= thr_safe) break;
        // a guess: accepted when the k-th with its band margin lies within it
        ++res.selects;
        const float kth = warp_kth32_lin(s, cnt, k, start);
        if (kth * (1.0f + 2.0f * kRelMargin) <= start) {
            kth_known = kth;
            break;
        }
    }
    if (!res.fail && cnt < k) res.fail = ALB_ERR_INVALID;
    if (res.fail) return true;
    if (QSPLIT) {
        // the float64 query is exactly its float32 split (f + l): rebuilt here rather than
        // held in registers through the search
        qx = (double)fx + (double)lx;
        qy = (double)fy + (double)ly;
        qz = (double)fz + (double)lz;
    }
    double rk2;
    if (REFINE) {
        rk2 = select_refined(m, s, 0, cnt, k, qx, qy, qz, tie_rec, res.clipped);
    } else {
        // float32 k-th; entries clearly below it are in, the band within the screening
        // margin around it is resolved exactly (refined keys when it is crowded)
        const float kth = kth_known >= 0.f ? kth_known : warp_kth32(s, 0, cnt, k);
        const float blo = kth * (1.0f - 2.0f * kRelMargin), bhi = kth * (1.0f + 2.0f * kRelMargin);
        int n_in = 0, n_band = 0;
#pragma unroll 1
        for (int base = 0; base < cnt; base += 32) {
            const int i = base + l;
            const bool valid = i < cnt;
            const float d = valid ? s.cd[i] : FLT_MAX;
            const uint32_t id = valid ? s.ci[i] : 0u;
            const bool in = valid && d < blo;
            const bool band = valid && d >= blo && d <= bhi;
            const unsigned bin = __ballot_sync(0xffffffffu, in);
            const unsigned bb = __ballot_sync(0xffffffffu, band);
            __syncwarp();
            if (in) s.ci[n_in + __popc(bin & lanemask_lt())] = id;
            if (band) {
                const int pos = n_band + __popc(bb & lanemask_lt());
                if (pos < kStack) s.stk[pos] = id;  // the stack is free after the search
            }
            n_in += __popc(bin);
            n_band += __popc(bb);
            __syncwarp();
        }
        if (n_band > kStack) {
            n_band = kStack;
            res.clipped = 1;
        }
        const int take = k - n_in;
        if (n_band <= kBand) {
            if (l < n_band) s.bi[l] = s.stk[l];
            __syncwarp();
            rk2 = rank_band(m, s, n_in, n_band, take, qx, qy, qz, tie_rec);
        } else {
#pragma unroll 1
            for (int j = l; j < n_band; j += 32) {
                const uint32_t id = s.stk[j];
                float hi, lo;
                point_dist2_df(fx, fy, fz, lx, ly, lz, m.a[id], hi, lo);
                s.cd[n_in + j] = hi;
                s.cl[n_in + j] = frac16(hi, lo);
                s.ci[n_in + j] = id;
            }
            __syncwarp();
            rk2 = select_refined(m, s, n_in, n_band, take, qx, qy, qz, tie_rec, res.clipped);
        }
    }
    res.rk2 = rk2;
    res.rkf = sqrt_to_f32(rk2);
    return true;
}

// ----------------------------------------------------------------------------------------
// per-neighbour weights (float32 restatement of the reference's energy multipliers)
// ----------------------------------------------------------------------------------------

// GGX Cook-Torrance, alb_sim/physics/reflection/microfacet_brdf.py:96-147, with
// wi = normalize(-d_map), wo = normalize(-d_query), n = +y.
ALB_DEVICE float ggx_weight(float a2, float f0, float wix, float wiy, float wiz, float wox, float woy, float woz) {
    float ni = rsqrtf(fmaf(wix, wix, fmaf(wiy, wiy, wiz * wiz)));
    wix *= ni; wiy *= ni; wiz *= ni;
    float n_wi = fminf(fmaxf(wiy, 0.f), 1.f);
    float n_wo = fminf(fmaxf(woy, 0.f), 1.f);
    if (!(n_wi > 0.f && n_wo > 0.f)) return 0.f;
    // Unnormalised half vector H = wi + wo. The reference's denominator
    // (a2 - 1) (n.h)^2 + 1 cancels near the specular peak; with h = H / |H| it equals
    // (Hx^2 + Hz^2 + a2 Hy^2) / |H|^2, a sum of non-negative terms that float32 keeps.
    float Hx = wix + wox, Hy = wiy + woy, Hz = wiz + woz;
    float t = fmaf(Hx, Hx, Hz * Hz);
    float H2 = fmaf(Hy, Hy, t);
    float den = 1.f, wi_h = 0.f;
    if (H2 > 0.f) {
        float inv = 1.f / H2;
        if (Hy > 0.f) den = fmaf(a2 * Hy, Hy, t) * inv;
        wi_h = fminf(fmaxf(fmaf(wix, Hx, fmaf(wiy, Hy, wiz * Hz)) * rsqrtf(H2), 0.f), 1.f);
    }
    float D = a2 / (3.14159265358979f * den * den + kEps32);
    float g1i = 2.f * n_wi / (n_wi + sqrtf(fmaf(1.f - a2, n_wi * n_wi, a2)));
    float g1o = 2.f * n_wo / (n_wo + sqrtf(fmaf(1.f - a2, n_wo * n_wo, a2)));
    float x = 1.f - wi_h;
    float x2 = x * x;
    float F = f0 + (1.f - f0) * (x2 * x2 * x);
    return (D * g1i * g1o * F) / (4.f * n_wi * n_wo + kEps32);
}

// Scatter weight: CDF mass of the angular bin of theta = acos(d_map . view),
// alb_sim/physics/scatter/energy.py:8-52 (view = normalize(-d_query)).
ALB_DEVICE int scatter_bin(const SceneDev& sc, int layer, float dx, float dy, float dz, float vx, float vy, float vz) {
    float n = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    float c = fmaf(dx, vx, fmaf(dy, vy, dz * vz)) * n;
    c = fminf(fmaxf(c, -1.f), 1.f);
    float th = acosf(c);
    int i = (int)((th - kEps32) / sc.layer_binw[layer]);
    return min(max(i, 0), ALB_PHASE_DIVISIONS - 1);
}
ALB_DEVICE float scatter_weight(const SceneDev& sc, int layer, float dx, float dy, float dz, float vx, float vy, float vz) {
    return __ldg(sc.layer_weight[layer] + scatter_bin(sc, layer, dx, dy, dz, vx, vy, vz));
}

// Adjoint (extension): d ln(ggx_weight) / d(alpha^2), the same vectors as ggx_weight:
// 1/a2 - 2 Hy^2 / (|H|^2 den) * pi den^2 / (pi den^2 + eps) from the distribution term and
// -(1 - n^2) / (2 s (n + s)), s = sqrt((1 - a2) n^2 + a2), from each Smith G1 factor; the
// Fresnel term has no a2.
ALB_DEVICE float ggx_dlog_da2(float a2, float wix, float wiy, float wiz, float wox, float woy, float woz) {
    float ni = rsqrtf(fmaf(wix, wix, fmaf(wiy, wiy, wiz * wiz)));
    wix *= ni; wiy *= ni; wiz *= ni;
    float n_wi = fminf(fmaxf(wiy, 0.f), 1.f);
    float n_wo = fminf(fmaxf(woy, 0.f), 1.f);
    if (!(n_wi > 0.f && n_wo > 0.f)) return 0.f;
    float Hx = wix + wox, Hy = wiy + woy, Hz = wiz + woz;
    float t = fmaf(Hx, Hx, Hz * Hz);
    float H2 = fmaf(Hy, Hy, t);
    float d = 1.f / a2;
    if (H2 > 0.f && Hy > 0.f) {
        float den = fmaf(a2 * Hy, Hy, t) / H2;
        // D = a2 / (pi den^2 + eps): the epsilon takes the share eps / (pi den^2 + eps) of
        // the denominator (about 0.6% at the specular peak for a2 = 0.0025)
        float pd2 = 3.14159265358979f * den * den;
        d -= 2.f * (Hy * Hy / H2) / den * (pd2 / (pd2 + kEps32));
    }
    float si = sqrtf(fmaf(1.f - a2, n_wi * n_wi, a2)), so = sqrtf(fmaf(1.f - a2, n_wo * n_wo, a2));
    d -= (1.f - n_wi * n_wi) / (2.f * si * (n_wi + si));
    d -= (1.f - n_wo * n_wo) / (2.f * so * (n_wo + so));
    return d;
}

// float32 -> 128-bit fixed point (64 fractional bits), integer ops only.
ALB_DEVICE Fix128 f32_to_fix(float v) {
    Fix128 r{0ull, 0ll};
    uint32_t b = __float_as_uint(v);
    uint32_t ex = (b >> 23) & 0xffu;
    if (ex == 0u || ex == 255u) return r;  // zero / subnormal / inf / nan contribute nothing
    uint64_t mant = (uint64_t)((b & 0x7fffffu) | 0x800000u);
    int sh = (int)ex - 150 + 64;  // value * 2^64 = mant * 2^sh
    uint64_t lo = 0ull, hi = 0ull;
    if (sh > 86) {
        lo = ~0ull;
        hi = 0x7fffffffffffffffull;
    } else if (sh >= 64) {
        hi = mant << (sh - 64);
    } else if (sh > 40) {
        lo = mant << sh;
        hi = mant >> (64 - sh);
    } else if (sh >= 0) {
        lo = mant << sh;
    } else if (sh > -24) {
        lo = mant >> (-sh);
    }
    if (b & 0x80000000u) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    r.lo = lo;
    r.hi = (long long)hi;
    return r;
}

// Per-CTA shared-memory cache of waveform bins: direct-mapped on the bin index, a slot is
// claimed once by CAS on its tag; hits are exact 128-bit integer adds in shared memory,
// misses go to global memory. Flushed once when the CTA finishes. The sum is integer, so
// the split between cache and global memory cannot change the result.
constexpr int kBinCache = 256;
struct BinCache {
    int tag[kBinCache];
    unsigned long long lo[kBinCache];
    unsigned long long hi[kBinCache];
};

ALB_DEVICE void bin_add(BinCache& bc, const Accum& acc, int channel, int bin, const Fix128& f) {
    int slot = bin & (kBinCache - 1);
    int t = bc.tag[slot];
    if (t != bin && t == -1) {
        int old = atomicCAS(&bc.tag[slot], -1, bin);
        t = (old == -1) ? bin : old;
    }
    if (t == bin) {
        fix_atomic_add(&bc.lo[slot], &bc.hi[slot], f);
    } else {
        uint64_t o = (uint64_t)channel * acc.nbins + bin;
        fix_atomic_add(acc.wf_lo + o, acc.wf_hi + o, f);
    }
}

// Extension (no counterpart in the reference): every record within the fixed radius R of
// the query, visited in any order. Screening as in the k-NN search; points within the
// float32 error band of R are decided on their float64 distance. visit(record) runs on the
// lanes holding admitted records.
template <class F>
ALB_DEVICE void warp_radius_visit(const MapDev& m, WarpSmem& s, double qx, double qy, double qz, float fx, float fy,
                                  float fz, float lx, float ly, float lz, double R, F&& visit, KnnResult& res) {
    const int l = lane_id();
    const double R2 = R * R;
    const float thr = __double2float_ru(R2) * (1.0f + 2.0f * kRelMargin);
    const float lo_band = __double2float_rd(R2) * (1.0f - 2.0f * kRelMargin);
    res.leaves = res.nodes = res.selects = res.clipped = res.fail = 0;
    res.rk2 = R2;
    res.rkf = (float)R;
    if (m.nlevels <= 0) return;  // an empty map contributes nothing
    int sp = 0;
    {
        const int top = m.nlevels - 1;
        bool ok = false;
        if ((uint64_t)l < m.lvl_cnt[top])
            ok = box_dist2(fx, fy, fz, lx, ly, lz, m.box_lo[m.lvl_off[top] + l], m.box_hi[m.lvl_off[top] + l]) <= thr;
        const unsigned b = __ballot_sync(0xffffffffu, ok);
        if (ok) s.stk[sp + __popc(b & lanemask_lt())] = ((uint32_t)top << 29) | (uint32_t)l;
        sp += __popc(b);
        __syncwarp();
    }
    // every box is pushed at most once, so the box count bounds the loop
    const uint64_t boxes = m.lvl_off[m.nlevels - 1] + m.lvl_cnt[m.nlevels - 1];
    uint64_t guard = 0;
    while (sp > 0) {
        if (++guard > boxes) {
            res.fail = ALB_ERR_ITER_CAP;
            break;
        }
        --sp;
        const uint32_t e = s.stk[sp];
        __syncwarp();
        const int lev = (int)(e >> 29);
        const uint32_t node = e & 0x1fffffffu;
        if (lev == 0) {
            ++res.leaves;
            const uint64_t r = (uint64_t)node * 32 + l;
            bool in = false;
            if (r < m.n) {
                const float4 p = m.a[r];
                const float d = point_dist2(fx, fy, fz, lx, ly, lz, p);
                in = d < lo_band || (d <= thr && point_dist2_f64(qx, qy, qz, p) <= R2);
            }
            if (in) visit((uint32_t)r);
        } else {
            ++res.nodes;
            const int cl = lev - 1;
            const uint64_t c = (uint64_t)node * 32 + l;
            bool ok = false;
            if (c < m.lvl_cnt[cl])
                ok = box_dist2(fx, fy, fz, lx, ly, lz, m.box_lo[m.lvl_off[cl] + c], m.box_hi[m.lvl_off[cl] + c]) <= thr;
            const unsigned b = __ballot_sync(0xffffffffu, ok);
            if (ok) s.stk[sp + __popc(b & lanemask_lt())] = ((uint32_t)cl << 29) | (uint32_t)c;
            sp += __popc(b);
            __syncwarp();
        }
    }
}

// Adjoint (extension): one neighbour's c (s_query + s_record + d ln w / d theta) into the
// Jacobian for theta = a, b, g, albedo, roughness (128-bit fixed point, global atomics).
template <int CHANNEL>
ALB_DEVICE void jac_add(const SceneDev& sc, const MapDev& m, const Accum& acc, int layer, int bin, uint32_t idx,
                        float c, float4 sq, float4 pb, float vx, float vy, float vz) {
    const float4 sp = m.sco ? m.sco[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    float d[kJacParams];
    d[0] = sq.x + sp.x;
    d[1] = sq.y + sp.y;
    d[2] = sq.z + sp.z;
    d[3] = sq.w + sp.w;
    d[4] = 0.f;
    if (CHANNEL == ALB_SCATTER && sc.layer_dlw_g[layer])
        d[2] += __ldg(sc.layer_dlw_g[layer] + scatter_bin(sc, layer, pb.x, pb.y, pb.z, vx, vy, vz));
    if (CHANNEL == ALB_BOTTOM_REFLECTION) d[3] += sc.inv_albedo;
    if (CHANNEL == ALB_SURFACE_REFLECTION) d[4] = sc.dla2_drough * ggx_dlog_da2(sc.ggx_a2, -pb.x, -pb.y, -pb.z, vx, vy, vz);
#pragma unroll
    for (int p = 0; p < kJacParams; ++p) {
        const float v = c * d[p];
        if (v != 0.f) {
            const uint64_t o = ((uint64_t)p * ALB_CHANNELS + CHANNEL) * acc.nbins + bin;
            fix_atomic_add(acc.jac_lo + o, acc.jac_hi + o, f32_to_fix(v));
        }
    }
}

// accumulate_to_heatmap (alb_sim/math/accumulate_heatmap.py:6-61) for one neighbour
ALB_DEVICE void heat_add(const SceneDev& sc, const MapDev& m, const Accum& acc, uint32_t idx, float c) {
    const float4 fw = m.fwi[idx], sf = m.sfi[idx];
    const Fix128 f = f32_to_fix(c);
    if (fw.x == fw.x) {
        long long xi = (long long)(((double)fw.x - sc.wc[0] + sc.hm_wext) / sc.hm_wbin);
        long long zi = (long long)(((double)fw.z - sc.wc[2] + sc.hm_wext) / sc.hm_wbin);
        if (xi >= 0 && xi < sc.hm_bins && zi >= 0 && zi < sc.hm_bins)
            fix_atomic_add(acc.hw_lo + xi * sc.hm_bins + zi, acc.hw_hi + xi * sc.hm_bins + zi, f);
    }
    if (sf.x == sf.x) {
        long long xi = (long long)(((double)sf.x - sc.fc[0] + sc.hm_fext) / sc.hm_fbin);
        long long zi = (long long)(((double)sf.z - sc.fc[2] + sc.hm_fext) / sc.hm_fbin);
        if (xi >= 0 && xi < sc.hm_bins && zi >= 0 && zi < sc.hm_bins)
            fix_atomic_add(acc.hf_lo + xi * sc.hm_bins + zi, acc.hf_hi + xi * sc.hm_bins + zi, f);
    }
}

// MODE: kModeKnn (the reference's estimator without heatmaps, the hot path),
// kModeKnnAdjoint (k-NN with the Jacobian, and heatmaps when set), kModeRadius (fixed
// radius; Jacobian and heatmaps when their accumulators are set), kModeKnnHeat (k-NN with
// the sampled heatmaps, the reference's default). Separate instantiations keep code a run
// never executes out of its instruction stream: the kernel is bound by instruction issue
// and fetch.
constexpr int kModeKnn = 0, kModeKnnAdjoint = 1, kModeRadius = 2, kModeKnnHeat = 3;

template <int CHANNEL, int MODE>
__global__ void __launch_bounds__(kGatherWarps * 32, kGatherBlocksPerSM) k_gather(SceneDev sc, MapDev m, QueryDev q, Accum acc, int k,
                                                              int* err) {
    __shared__ WarpSmem smem[kGatherWarps];
    __shared__ BinCache bc;
    for (int i = threadIdx.x; i < kBinCache; i += blockDim.x) {
        bc.tag[i] = -1;
        bc.lo[i] = 0ull;
        bc.hi[i] = 0ull;
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, l = lane_id();
    WarpSmem& s = smem[w];
    const uint64_t warps = (uint64_t)gridDim.x * kGatherWarps;
    constexpr int kChunk = CHANNEL == ALB_SCATTER ? kQueryChunkScatter : kQueryChunk;
    const uint64_t chunks = (q.n + kChunk - 1) / kChunk;
    bool failed = false;
    // search counters accumulate in the warp's shared memory, not in registers held through
    // every search
    if (l < 5) s.st[l] = 0ull;
    __syncwarp();
    for (uint64_t ch = (uint64_t)blockIdx.x * kGatherWarps + w; ch < chunks && !failed; ch += warps) {
        const uint64_t q_end = min((ch + 1) * kChunk, q.n);
        bool have_prev = false;  // s.ci[0 .. k) holds the previous query's neighbours
        for (uint64_t qi = ch * kChunk; qi < q_end; ++qi) {
            uint64_t src = q.perm ? q.perm[qi] : qi;
            const float4 qa = q.a[src], qc = q.c[src];
            if (MODE == kModeRadius) {
                const float4 qb = q.b[src];
                const double qx = (double)qa.x + (double)qc.x, qy = (double)qa.y + (double)qc.y,
                             qz = (double)qa.z + (double)qc.z;
                // extension: every record within the fixed radius contributes at once
                KnnResult r;
                const float Es = qa.w, ts = qb.w;
                const float R = (float)sc.radius;
                const float norm = (CHANNEL == ALB_SCATTER) ? 1.0f / ((4.0f / 3.0f) * 3.14159265358979f * R * R * R)
                                                            : 1.0f / (3.14159265358979f * R * R);
                const float vinv = rsqrtf(fmaf(qb.x, qb.x, fmaf(qb.y, qb.y, qb.z * qb.z)));
                const float vx = -qb.x * vinv, vy = -qb.y * vinv, vz = -qb.z * vinv;
                float wconst = 0.f;
                if (CHANNEL == ALB_BOTTOM_REFLECTION) wconst = (float)(sc.floor_albedo / kPi) * fmaxf(0.f, -qb.y);
                if (CHANNEL == ALB_SURFACE_TRANSMISSION_UP) wconst = (float)(sc.surface_albedo / kPi);
                const int layer = (CHANNEL == ALB_SCATTER) ? layer_of(sc, qy) : 0;
                const float4 sq = q.s ? q.s[src] : make_float4(0.f, 0.f, 0.f, 0.f);
                warp_radius_visit(m, s, qx, qy, qz, qa.x, qa.y, qa.z, qc.x, qc.y, qc.z, sc.radius,
                    [&](uint32_t idx) {
                        const float4 pb = m.b[idx];
                        float w;
                        if (CHANNEL == ALB_BOTTOM_REFLECTION || CHANNEL == ALB_SURFACE_TRANSMISSION_UP) w = wconst;
                        else if (CHANNEL == ALB_SCATTER) w = scatter_weight(sc, layer, pb.x, pb.y, pb.z, vx, vy, vz);
                        else w = ggx_weight(sc.ggx_a2, (float)sc.f0, -pb.x, -pb.y, -pb.z, vx, vy, vz);
                        const float c = ((Es * m.a[idx].w) * norm) * w;
                        const int bin = (int)((ts + pb.w) / (float)sc.mult) - (int)sc.gate_lo;
                        if (bin >= 0 && bin < acc.nbins) {
                            bin_add(bc, acc, CHANNEL, bin, f32_to_fix(c));
                            if (acc.jac_lo) jac_add<CHANNEL>(sc, m, acc, layer, bin, idx, c, sq, pb, vx, vy, vz);
                        } else if (!sc.gated) {
                            atomicCAS(err, 0, ALB_ERR_CAPACITY);
                        }
                        if (acc.hw_lo && m.fwi) heat_add(sc, m, acc, idx, c);
                    },
                    r);
                if (r.fail) {
                    if (l == 0) atomicCAS(err, 0, r.fail);
                    failed = true;
                    break;
                }
                if (l == 0) {
                    s.st[0] += r.leaves;
                    s.st[1] += r.nodes;
                    s.st[3] += 1;
                    s.st[4] += r.clipped;
                }
                if (q.rk_out && l == 0) q.rk_out[src] = sc.radius;
                __syncwarp();
                continue;
            }
            float thr_safe = FLT_MAX, thr0 = FLT_MAX;
            if (have_prev) {
                // the float32 screening error (below 2^-21) is far inside the 2^-14 inflation
                unsigned mx = 0u;
                float4 pn = l < k ? m.a[s.ci[l]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1  // rolled: the kernel is bound by instruction fetch, and these loops run 4 times
                for (int j = l; j < k; j += 32) {
                    const float4 p = pn;
                    if (j + 32 < k) pn = m.a[s.ci[j + 32]];  // in flight during this neighbour
                    const float d = point_dist2(qa.x, qa.y, qa.z, qc.x, qc.y, qc.z, p);
                    mx = max(mx, __float_as_uint(d));  // non-negative floats order like their bits
                }
                const float t = __uint_as_float(__reduce_max_sync(0xffffffffu, mx)) * (1.f + 1.f / 16384.f);
                if (t < 1.0e37f) thr_safe = t;
                // The safe bound is the farthest of the previous query's neighbours, about
                // twice the k-th distance here (the sorted queries are about one k-th
                // distance apart): eight times the ball. Consecutive k-th distances differ by
                // less than 20% for 99.7% of the scatter map's sorted queries, so the first
                // search uses (1.2 r_prev)^2 and is redone under the safe bound when that
                // does not hold. Planar maps keep the safe bound.
                thr0 = (CHANNEL == ALB_SCATTER) ? fminf(thr_safe, s.prev_rk2 * kGuessWiden2) : thr_safe;
            }
            KnnResult r;
            if (!warp_knn<CHANNEL != ALB_SCATTER, true>(m, s, k, 0.0, 0.0, 0.0, qa.x, qa.y, qa.z, qc.x, qc.y, qc.z,
                                                         thr0, thr_safe, m.b, r)) {
                if (l == 0) atomicCAS(err, 0, ALB_ERR_TOO_FEW);
                failed = true;
                break;
            }
            if (r.fail) {  // no valid neighbour set: report it and stop this warp's work
                if (l == 0) atomicCAS(err, 0, r.fail);
                failed = true;
                break;
            }
            // the query's direction and time, and its float64 depth, are needed from here on
            const float4 qb = q.b[src];
            const double qy = (double)qa.y + (double)qc.y;
            have_prev = true;
            if (l == 0) s.prev_rk2 = (float)r.rk2;  // read after the next query's __syncwarp
            if (q.rk_out && l == 0) q.rk_out[src] = sqrt(r.rk2);
            if (l == 0) {
                s.st[0] += r.leaves;
                s.st[1] += r.nodes;
                s.st[2] += r.selects;
                s.st[3] += 1;
                s.st[4] += r.clipped;
            }
            if (r.retried && l == 0 && q.retries) atomicAdd(q.retries, 1ull);  // rare: no register kept
            const float Es = qa.w, ts = qb.w;
            const float rk = r.rkf;
            float norm;
            if (CHANNEL == ALB_SCATTER) norm = 1.0f / ((4.0f / 3.0f) * 3.14159265358979f * rk * rk * rk);
            else norm = 1.0f / (3.14159265358979f * rk * rk);
            // query-constant pieces
            float vinv = rsqrtf(fmaf(qb.x, qb.x, fmaf(qb.y, qb.y, qb.z * qb.z)));
            float vx = -qb.x * vinv, vy = -qb.y * vinv, vz = -qb.z * vinv;  // normalize(-d_query)
            float wconst = 0.f;
            if (CHANNEL == ALB_BOTTOM_REFLECTION) wconst = (float)(sc.floor_albedo / kPi) * fmaxf(0.f, -qb.y);
            if (CHANNEL == ALB_SURFACE_TRANSMISSION_UP) wconst = (float)(sc.surface_albedo / kPi);
            // WaterModel.scatter_energy picks the layer of the query depth (water.py:418-447)
            const int layer = (CHANNEL == ALB_SCATTER) ? layer_of(sc, qy) : 0;
            float4 sq = make_float4(0.f, 0.f, 0.f, 0.f);
            if (MODE == kModeKnnAdjoint && q.s) sq = q.s[src];
            // the next neighbour's record is loaded while this one is weighted
            uint32_t idx_n = l < k ? s.ci[l] : 0u;
            float4 pb_n = make_float4(0.f, 0.f, 0.f, 0.f);
            float e_n = 0.f;
            if (l < k) {
                pb_n = m.b[idx_n];
                e_n = m.a[idx_n].w;
            }
#pragma unroll 1
            for (int j = l; j < k; j += 32) {
                const uint32_t idx = idx_n;
                const float4 pb = pb_n;
                const float Ep = e_n;
                if (j + 32 < k) {
                    idx_n = s.ci[j + 32];
                    pb_n = m.b[idx_n];
                    e_n = m.a[idx_n].w;
                }
                float w;
                if (CHANNEL == ALB_BOTTOM_REFLECTION || CHANNEL == ALB_SURFACE_TRANSMISSION_UP) w = wconst;
                else if (CHANNEL == ALB_SCATTER) w = scatter_weight(sc, layer, pb.x, pb.y, pb.z, vx, vy, vz);
                else w = ggx_weight(sc.ggx_a2, (float)sc.f0, -pb.x, -pb.y, -pb.z, vx, vy, vz);
                const float c = ((Es * Ep) * norm) * w;
                const int bin = (int)((ts + pb.w) / (float)sc.mult) - (int)sc.gate_lo;
                if (bin >= 0 && bin < acc.nbins) {
                    bin_add(bc, acc, CHANNEL, bin, f32_to_fix(c));
                    if (MODE == kModeKnnAdjoint && acc.jac_lo)
                        jac_add<CHANNEL>(sc, m, acc, layer, bin, idx, c, sq, pb, vx, vy, vz);
                } else if (!sc.gated) {
                    atomicCAS(err, 0, ALB_ERR_CAPACITY);
                }
            }
            if (MODE != kModeKnn && acc.hw_lo && m.fwi) {
                // accumulate_to_heatmap, alb_sim/math/accumulate_heatmap.py:6-61 (a separate,
                // non-unrolled pass: heatmaps are off in production runs)
#pragma unroll 1
                for (int j = l; j < k; j += 32) {
                    const uint32_t idx = s.ci[j];
                    const float4 pb = m.b[idx];
                    float w;
                    if (CHANNEL == ALB_BOTTOM_REFLECTION || CHANNEL == ALB_SURFACE_TRANSMISSION_UP) w = wconst;
                    else if (CHANNEL == ALB_SCATTER) w = scatter_weight(sc, layer, pb.x, pb.y, pb.z, vx, vy, vz);
                    else w = ggx_weight(sc.ggx_a2, (float)sc.f0, -pb.x, -pb.y, -pb.z, vx, vy, vz);
                    heat_add(sc, m, acc, idx, ((Es * m.a[idx].w) * norm) * w);
                }
            }
            __syncwarp();
        }
    }
    if (l == 0) {
        if (q.stats && s.st[3]) {
            atomicAdd(q.stats + 0, s.st[0]);
            atomicAdd(q.stats + 1, s.st[1]);
            atomicAdd(q.stats + 2, s.st[2]);
            atomicAdd(q.stats + 3, s.st[3]);
        }
        if (q.inexact && s.st[4]) atomicAdd(q.inexact, s.st[4]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBinCache; i += blockDim.x) {
        int t = bc.tag[i];
        if (t >= 0) {
            uint64_t o = (uint64_t)CHANNEL * acc.nbins + t;
            Fix128 f{bc.lo[i], (long long)bc.hi[i]};
            fix_atomic_add(acc.wf_lo + o, acc.wf_hi + o, f);
        }
    }
}

// Standalone KDTree.query(x, k): sorted indices and float64 distances.
__global__ void __launch_bounds__(kGatherWarps * 32) k_knn(MapDev m, const double* __restrict__ qs, uint64_t nq,
                                                           int k, int32_t* out_idx, double* out_dist, int* err) {
    __shared__ WarpSmem smem[kGatherWarps];
    const int w = threadIdx.x >> 5, l = lane_id();
    WarpSmem& s = smem[w];
    const uint64_t warps = (uint64_t)gridDim.x * kGatherWarps;
    for (uint64_t qi = (uint64_t)blockIdx.x * kGatherWarps + w; qi < nq; qi += warps) {
        double qx = qs[3 * qi], qy = qs[3 * qi + 1], qz = qs[3 * qi + 2];
        KnnResult r;
        const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
        int why = 0;
        if (!warp_knn<true>(m, s, k, qx, qy, qz, fx, fy, fz, (float)(qx - (double)fx), (float)(qy - (double)fy),
                            (float)(qz - (double)fz), FLT_MAX, FLT_MAX, nullptr, r))
            why = ALB_ERR_TOO_FEW;
        else if (r.fail)
            why = r.fail;
        if (why) {
            // a query without an answer gets index -1 and distance NaN in all its k slots,
            // so no slot is left holding whatever the caller's buffer held before
            if (l == 0) atomicCAS(err, 0, why);
            for (int j = l; j < k; j += 32) {
                out_idx[qi * k + j] = -1;
                out_dist[qi * k + j] = __longlong_as_double(0x7ff8000000000000ll);
            }
            __syncwarp();
            continue;
        }
        // float64 distances of the k neighbours, then rank-sort them (k <= kMaxK)
        for (int j = l; j < k; j += 32) {
            uint32_t idx = s.ci[j];
            double d = point_dist2_f64(qx, qy, qz, m.a[idx]);
            int rank = 0;
            for (int t = 0; t < k; ++t) {
                uint32_t it = s.ci[t];
                double dt = point_dist2_f64(qx, qy, qz, m.a[it]);
                rank += (dt < d || (dt == d && it < idx)) ? 1 : 0;
            }
            out_idx[qi * k + rank] = (int32_t)idx;
            out_dist[qi * k + rank] = sqrt(d);
        }
        __syncwarp();
    }
}

static unsigned gather_blocks(uint64_t nq) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t want = (nq + kGatherWarps - 1) / kGatherWarps;
    uint64_t cap = (uint64_t)sms * 16;
    return (unsigned)(want < cap ? (want ? want : 1) : cap);
}

template <int MODE>
static void launch_gather_mode(const MapDev& map, const QueryDev& q, int channel, const SceneDev& sc, const Accum& acc,
                               int* err, unsigned blocks, int k, cudaStream_t st) {
    switch (channel) {
        case ALB_BOTTOM_REFLECTION:
            k_gather<ALB_BOTTOM_REFLECTION, MODE><<<blocks, kGatherWarps * 32, 0, st>>>(sc, map, q, acc, k, err);
            break;
        case ALB_SCATTER:
            k_gather<ALB_SCATTER, MODE><<<blocks, kGatherWarps * 32, 0, st>>>(sc, map, q, acc, k, err);
            break;
        case ALB_SURFACE_REFLECTION:
            k_gather<ALB_SURFACE_REFLECTION, MODE><<<blocks, kGatherWarps * 32, 0, st>>>(sc, map, q, acc, k, err);
            break;
        default:
            k_gather<ALB_SURFACE_TRANSMISSION_UP, MODE><<<blocks, kGatherWarps * 32, 0, st>>>(sc, map, q, acc, k, err);
            break;
    }
    note_launch();
}

void launch_gather(const SceneDev& sc, const MapDev& map, const QueryDev& q, int channel, const Accum& acc,
                   int* err, int* launches, cudaStream_t st) {
    if (q.n == 0) return;
    unsigned blocks = gather_blocks(q.n);
    int k = sc.k;
    if (sc.radius > 0.0) launch_gather_mode<kModeRadius>(map, q, channel, sc, acc, err, blocks, k, st);
    else if (acc.jac_lo) launch_gather_mode<kModeKnnAdjoint>(map, q, channel, sc, acc, err, blocks, k, st);
    else if (acc.hw_lo && map.fwi) launch_gather_mode<kModeKnnHeat>(map, q, channel, sc, acc, err, blocks, k, st);
    else launch_gather_mode<kModeKnn>(map, q, channel, sc, acc, err, blocks, k, st);
    if (launches) ++*launches;
}

void launch_knn(const MapDev& map, const double* queries, uint64_t nq, int k, int32_t* out_idx, double* out_dist,
                int* err, cudaStream_t st) {
    if (nq == 0) return;
    k_knn<<<gather_blocks(nq), kGatherWarps * 32, 0, st>>>(map, queries, nq, k, out_idx, out_dist, err);
    note_launch();
}

}  // namespace alb
