// Device-side building blocks shared by the tracer, map build and gather kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "albgpu.h"

#define ALB_HOST_DEVICE __host__ __device__ __forceinline__
#define ALB_DEVICE __device__ __forceinline__

namespace alb {

constexpr int kWarp = 32;
constexpr double kTwoPi = 6.283185307179586;   // 2 * np.pi as the reference forms it
constexpr double kPi = 3.141592653589793;
constexpr float kEps32 = 1.1920928955078125e-07f;  // np.finfo(np.float32).eps
constexpr int kMaxEventsPerPhoton = 1 << 22;    // device loop cap -> ALB_ERR_ITER_CAP

// Scene constants in __constant__ memory (one copy per loaded module).
struct SceneDev {
    double dt;
    int64_t total_steps;      // steps * sample_multiplier
    int64_t stop_step[2];     // per pass: steps traced (total_steps unless a gate ends earlier)
    int64_t nbins;            // 2 * steps, or the gate's length
    int64_t gate_lo;          // first timeline bin of the waveform (gated windows)
    int32_t gated;            // 1: bins outside the window are dropped, not an error
    int32_t pad_gate;
    int32_t mult;
    int32_t k;
    double ys, yf, v_air;
    double n_water, eta, f0;
    double floor_albedo, surface_albedo, roughness;
    double radius;            // extension: fixed gather radius (m), 0 = k nearest
    double slope_sigma;       // extension: Gaussian surface-slope std (0 = flat surface)
    float floor_albedo32;
    float ggx_a2;             // (roughness^2)^2 as used by the GGX distribution
    double rot_d[9];          // float32 laser rotation, widened
    double div, fov, cos_fov, aperture, pulse_sigma32, eff_rate32;
    double rayleigh_sigma, rayleigh_mass;  // truncated-Rayleigh inverse CDF constants
    int32_t n_layers;
    int32_t heatmap;
    int32_t hm_bins;
    int32_t pad0;
    double hm_wext, hm_fext, hm_wbin, hm_fbin;
    double wc[3], fc[3];
    double layer_bottom[ALB_MAX_LAYERS];
    double layer_speed[ALB_MAX_LAYERS];
    float layer_alpha[ALB_MAX_LAYERS];
    float layer_ssa[ALB_MAX_LAYERS];
    float layer_binw[ALB_MAX_LAYERS];
    const double* layer_theta[ALB_MAX_LAYERS];
    const double* layer_cdf[ALB_MAX_LAYERS];
    const double* layer_slope[ALB_MAX_LAYERS];
    const float* layer_weight[ALB_MAX_LAYERS];
    // depth-profiled layers (layer_prof != 0): per-step speed, attenuation and albedo
    int32_t layer_prof[ALB_MAX_LAYERS];
    int32_t layer_lut_n[ALB_MAX_LAYERS];
    const float* layer_lut_z[ALB_MAX_LAYERS];
    const double* layer_lut_a[ALB_MAX_LAYERS];
    int32_t layer_nkind[ALB_MAX_LAYERS];
    int32_t layer_akind[ALB_MAX_LAYERS];
    double layer_n0[ALB_MAX_LAYERS], layer_n1[ALB_MAX_LAYERS];
    double layer_a0[ALB_MAX_LAYERS], layer_a1[ALB_MAX_LAYERS];
    double layer_h[ALB_MAX_LAYERS], layer_top32[ALB_MAX_LAYERS];
    // adjoint (extension): path scores for theta = (a, b, g) and the seafloor albedo
    int32_t adjoint;
    int32_t pad1;
    float adj_dla[ALB_MAX_LAYERS][3];  // d ln(alpha) / d theta
    float adj_dls[ALB_MAX_LAYERS][3];  // d ln(ssa) / d theta
    float layer_hg_g[ALB_MAX_LAYERS];  // HG asymmetry (0: not an HG layer)
    const float* layer_dlw_g[ALB_MAX_LAYERS];  // d ln(scatter weight) / dg per bin
    const float* layer_dsg[ALB_MAX_LAYERS];    // d ln(mass) / dg per sampling interval (nullable)
    float inv_albedo;                  // 1 / seafloor albedo (0 when the albedo is 0)
    float dla2_drough;                 // d (GGX alpha^2) / d roughness = 4 roughness^3
};

// Path score of one photon for theta = (a, b, g, seafloor albedo).
struct Score {
    float a, b, g, l;
};

// d ln p_HG(mu) / dg for p_HG(mu) = (1 - g^2) / (4 pi (1 + g^2 - 2 g mu)^1.5)
ALB_HOST_DEVICE float hg_dlogp_dg(float g, float mu) {
    return -2.f * g / (1.f - g * g) - 3.f * (g - mu) / (1.f + g * g - 2.f * g * mu);
}

// ---------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3", SC'11).
// ---------------------------------------------------------------------------------------
struct U4 {
    uint32_t x, y, z, w;
};

ALB_HOST_DEVICE void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

ALB_HOST_DEVICE U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(M0, c.x, hi0, lo0);
        mulhilo(M1, c.z, hi1, lo1);
        U4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// (x + 0.5) / 2^32: a double strictly inside (0, 1).
ALB_HOST_DEVICE double u01(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386963e-10; }

// ---------------------------------------------------------------------------------------
// 128-bit two's-complement fixed point with 64 fractional bits. Every contribution is
// converted exactly (up to truncation below 2^-64) and summed with integer atomics, so
// the waveform is independent of summation order and bit-identical run to run.
// ---------------------------------------------------------------------------------------
struct Fix128 {
    unsigned long long lo;
    long long hi;
};

ALB_DEVICE Fix128 to_fix128(double v) {
    Fix128 r{0ull, 0ll};
    if (!(v != 0.0) || !isfinite(v)) return r;
    bool neg = v < 0.0;
    double a = neg ? -v : v;
    int e;
    double m = frexp(a, &e);                        // a = m * 2^e, m in [0.5, 1)
    unsigned long long mant = (unsigned long long)ldexp(m, 53);  // 53-bit integer
    int sh = e - 53 + 64;                            // value * 2^64 = mant * 2^sh
    unsigned long long lo = 0ull, hi = 0ull;
    if (sh > 74 || sh <= -53) {
        if (sh > 74) { lo = ~0ull; hi = 0x7fffffffffffffffull; }  // saturate at 2^63
    } else if (sh >= 64) {
        hi = mant << (sh - 64);
    } else if (sh > 0) {
        lo = mant << sh;
        hi = mant >> (64 - sh);
    } else if (sh == 0) {
        lo = mant;
    } else {
        lo = mant >> (-sh);
    }
    if (neg) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    r.lo = lo;
    r.hi = (long long)hi;
    return r;
}

ALB_DEVICE void fix_add(Fix128& a, const Fix128& b) {
    unsigned long long lo = a.lo + b.lo;
    a.hi = a.hi + b.hi + (lo < a.lo ? 1 : 0);
    a.lo = lo;
}

// Atomic 128-bit add into (lo, hi) words: exact modulo 2^128, order independent.
ALB_DEVICE void fix_atomic_add(unsigned long long* lo_word, unsigned long long* hi_word,
                               const Fix128& v) {
    if (v.lo == 0ull && v.hi == 0ll) return;
    unsigned long long old = atomicAdd(lo_word, v.lo);
    unsigned long long carry = (old + v.lo < old) ? 1ull : 0ull;
    unsigned long long h = (unsigned long long)v.hi + carry;
    if (h) atomicAdd(hi_word, h);
}

ALB_HOST_DEVICE double fix_to_double(unsigned long long lo, long long hi) {
    // hi * 2^0 + lo * 2^-64 (two's complement over 128 bits)
    return (double)hi + (double)lo * 5.421010862427522e-20;
}

// ---------------------------------------------------------------------------------------
// Warp helpers
// ---------------------------------------------------------------------------------------
ALB_DEVICE unsigned lane_id() { return threadIdx.x & 31u; }

ALB_DEVICE unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-aggregated append: the active lanes with equal `key` share one atomicAdd on
// counters[key]; returns this lane's slot.
ALB_DEVICE unsigned long long warp_append(unsigned long long* counters, int key) {
    unsigned active = __activemask();
    unsigned same = __match_any_sync(active, key);
    int leader = __ffs(same) - 1;
    unsigned rank = __popc(same & lanemask_lt());
    unsigned long long base = 0ull;
    if ((int)lane_id() == leader) base = atomicAdd(counters + key, (unsigned long long)__popc(same));
    base = __shfl_sync(same, base, leader);
    return base + rank;
}

}  // namespace alb
