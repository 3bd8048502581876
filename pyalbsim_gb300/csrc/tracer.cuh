// Photon tracer: one thread per photon, event-jump form of the reference's fixed-step
// integrator (alb_sim/core/simulation.py:71-107, 220-570).
//
// The reference advances every photon by d * v * dt per step for steps * multiplier steps
// and dispatches on (y, y_next). Nothing happens to a photon between events except that
// its position moves linearly and, in water, its float32 optical depth grows by
// alpha * |step| each step. This tracer therefore jumps straight to the step at which the
// next event happens:
//   * plane crossings: smallest n with y0 + n * sv_y beyond the plane (float64);
//   * scatter: the first step at which the float32 running sum tau reaches tau*, found by
//     an exact emulation of tau <- fl32(fl64(tau) + inc) that advances one float32 binade
//     at a time (inside a binade the rounded increment is constant);
//   * layer changes (multi-layer water): the first step starting in another layer.
// Event handling restates the reference's handlers: handle_water :328-373,
// handle_enter :375-431, handle_exit :433-502, handle_seafloor :504-570.
#pragma once

#include "device_common.cuh"

namespace alb {

constexpr int kQueryBottom = 0, kQueryScatter = 1, kQuerySurface = 2;

struct TraceOut {
    // forward photon-map records, per channel
    float4* rec_a[ALB_CHANNELS];  // x, y, z, energy
    float4* rec_b[ALB_CHANNELS];  // dx, dy, dz, time (integrator step)
    float4* rec_fwi[ALB_CHANNELS];  // nullable: first-water / seafloor interaction points
    float4* rec_sfi[ALB_CHANNELS];
    uint32_t* rec_id[ALB_CHANNELS];  // nullable
    float4* rec_sco[ALB_CHANNELS];   // adjoint path scores (nullable)
    unsigned long long* rec_count;   // [ALB_CHANNELS], cumulative over forward calls
    unsigned long long rec_cap[ALB_CHANNELS];
    // backward gather queries, per kind (bottom, scatter, surface)
    float4* q_a[3];  // x_hi, y_hi, z_hi, energy
    float4* q_b[3];  // dx, dy, dz, time
    float4* q_c[3];  // x_lo, y_lo, z_lo, 0   (x = x_hi + x_lo to ~1e-14)
    uint32_t* q_id[3];
    float4* q_s[3];  // adjoint path scores (nullable)
    unsigned long long* q_count;  // [3]
    unsigned long long q_cap[3];
    // per-photon final states (nullable)
    double* ex_pos;
    double* ex_dir;
    float* ex_f;  // energy, tau, tau_target, time, fwi[3], sfi[3] (10 per photon)
    // scatter-radius heatmap counts (forward, nullable)
    unsigned int* hm_radius;
    int* err;                      // first error code raised on the device
    unsigned long long* stats;     // [0] events, [1] photons finished
};

struct Ph {
    double px, py, pz;
    double dx, dy, dz;
    float E, tau, taut, t0;
    float fwi[3], sfi[3];
    int64_t s;
    Score sc;  // adjoint: d ln(p E) / d (a, b, g, albedo) of the path so far
};

// Adjoint score updates (extension). Free paths: tau grows by alpha |step| per step and a
// scatter happens where it reaches an Exp(1) target, so the path density carries
// alpha e^(-tau) per scatter and e^(-tau) per survival: an optical-depth increment dtau in
// layer L adds -dtau d ln(alpha_L)/d theta; a scatter adds +d ln(alpha_L)/d theta for its
// density and d ln(ssa_L)/d theta for its energy factor; HG sampling adds
// d ln p_HG(mu)/dg; a seafloor reflection adds 1/albedo.
ALB_DEVICE void score_tau(const SceneDev& sc, Score& s, int L, float dtau) {
    s.a = fmaf(-dtau, sc.adj_dla[L][0], s.a);
    s.b = fmaf(-dtau, sc.adj_dla[L][1], s.b);
    s.g = fmaf(-dtau, sc.adj_dla[L][2], s.g);
}
ALB_DEVICE void score_scatter_density(const SceneDev& sc, Score& s, int L) {
    s.a += sc.adj_dla[L][0];
    s.b += sc.adj_dla[L][1];
    s.g += sc.adj_dla[L][2];
}
// An HG angle is drawn from the tabulated CDF: its score is the g-derivative of the log-mass
// of the table interval it fell in (`interval`, from the CDF search or the angle); the
// analytic d ln p_HG(mu)/dg only when the scene carries no such table.
ALB_DEVICE void score_scatter_after(const SceneDev& sc, Score& s, int L, float mu, int interval) {
    s.a += sc.adj_dls[L][0];
    s.b += sc.adj_dls[L][1];
    s.g += sc.adj_dls[L][2];
    if (sc.layer_hg_g[L] != 0.f)
        s.g += sc.layer_dsg[L] ? __ldg(sc.layer_dsg[L] + interval) : hg_dlogp_dg(sc.layer_hg_g[L], mu);
}

// Table interval of an angle drawn by the float32 tracer (from the angle: interval i holds
// (theta_{i-1}, theta_i] on the uniform angle grid).
ALB_DEVICE int sample_interval_of_angle(const SceneDev& sc, int L, float th) {
    const double t0 = sc.layer_theta[L][0], dt = sc.layer_theta[L][1] - t0;
    const int i = (int)ceil(((double)th - t0) / dt);
    return min(max(i, 0), ALB_PHASE_DIVISIONS - 1);
}

ALB_DEVICE void set_err(int* err, int code) { atomicCAS(err, 0, code); }

// ----------------------------------------------------------------------------------------
// Variate sources
// ----------------------------------------------------------------------------------------

// Counter-based: photon `pid` of pass `pass` draws block j from Philox(ctr = {j, pid_lo,
// pid_hi, pass}, key = seed).
struct PhiloxSrc {
    uint32_t k0, k1, plo, phi, pass, ctr;
    ALB_DEVICE U4 block() {
        U4 c{ctr, plo, phi, pass};
        ++ctr;
        return philox4x32_10(c, k0, k1);
    }
};

// Replay: the photon's recorded variates in the reference's draw order.
struct ReplaySrc {
    const double* v;
    const float* tau;
    int64_t pos, end;
    int* err;
    ALB_DEVICE double next() {
        if (pos < end) return v[pos++];
        set_err(err, ALB_ERR_REPLAY);
        return 0.5;
    }
    ALB_DEVICE float next_tau() {
        if (pos < end) return tau[pos++];
        set_err(err, ALB_ERR_REPLAY);
        return 1.0f;
    }
};

// -log(float32(u)) as a float32, through a float64 log (precise form shared with the oracle).
ALB_DEVICE float tau_from_uniform(double u) {
    float f = __double2float_rn(u);
    return __double2float_rn(-log((double)f));
}

// Forward emission variates: theta (truncated Rayleigh), phi, pulse offset (s).
ALB_DEVICE void draw_emit_fwd(const SceneDev& sc, PhiloxSrc& s, double& th, double& ph, double& pulse) {
    U4 b = s.block();
    th = sc.rayleigh_sigma * sqrt(-2.0 * log(1.0 - u01(b.x) * sc.rayleigh_mass));
    ph = kTwoPi * u01(b.y);
    pulse = sc.pulse_sigma32 * (sqrt(-2.0 * log(u01(b.z))) * cos(kTwoPi * u01(b.w)));
}
ALB_DEVICE void draw_emit_fwd(const SceneDev&, ReplaySrc& s, double& th, double& ph, double& pulse) {
    th = s.next();
    ph = s.next();
    pulse = s.next();
}

// Backward emission variates: disk (xi1, xi2), cone (z, phi).
ALB_DEVICE void draw_emit_bwd(const SceneDev& sc, PhiloxSrc& s, double& x1, double& x2, double& z, double& ph) {
    U4 b = s.block();
    x1 = u01(b.x);
    x2 = u01(b.y);
    z = sc.cos_fov + (1.0 - sc.cos_fov) * u01(b.z);
    ph = kTwoPi * u01(b.w);
}
ALB_DEVICE void draw_emit_bwd(const SceneDev&, ReplaySrc& s, double& x1, double& x2, double& z, double& ph) {
    x1 = s.next();
    x2 = s.next();
    z = s.next();
    ph = s.next();
}

ALB_DEVICE void draw_scatter(PhiloxSrc& s, double& uth, double& phi, float& taut) {
    U4 b = s.block();
    uth = u01(b.x);
    phi = kTwoPi * u01(b.y);
    taut = tau_from_uniform(u01(b.z));
}
ALB_DEVICE void draw_scatter(ReplaySrc& s, double& uth, double& phi, float& taut) {
    uth = s.next();
    phi = s.next();
    taut = s.next_tau();
}

ALB_DEVICE float draw_tau(PhiloxSrc& s) { return tau_from_uniform(u01(s.block().x)); }
ALB_DEVICE float draw_tau(ReplaySrc& s) { return s.next_tau(); }

ALB_DEVICE double draw_uniform(PhiloxSrc& s) { return u01(s.block().x); }
ALB_DEVICE double draw_uniform(ReplaySrc& s) { return s.next(); }

// Three standard normals (Box-Muller on Philox; raw normals on replay).
ALB_DEVICE void draw_normals(PhiloxSrc& s, double& n0, double& n1, double& n2) {
    U4 b = s.block();
    double r0 = sqrt(-2.0 * log(u01(b.x)));
    double a0 = kTwoPi * u01(b.y);
    double r1 = sqrt(-2.0 * log(u01(b.z)));
    double a1 = kTwoPi * u01(b.w);
    n0 = r0 * cos(a0);
    n1 = r0 * sin(a0);
    n2 = r1 * cos(a1);
}
ALB_DEVICE void draw_normals(ReplaySrc& s, double& n0, double& n1, double& n2) {
    n0 = s.next();
    n1 = s.next();
    n2 = s.next();
}

// ----------------------------------------------------------------------------------------
// Geometry helpers (float64, operation order of the reference's NumPy expressions)
// ----------------------------------------------------------------------------------------

ALB_DEVICE int layer_of(const SceneDev& sc, double y) {
    // depth = (y - y_surface) * -1; layer = searchsorted(cumulative, depth, 'right'),
    // clipped to the last layer (alb_sim/physics/models/water.py:288-304).
    double depth = -(y - sc.ys);
    int i = 0;
    while (i < sc.n_layers && !(sc.layer_bottom[i] > depth)) ++i;
    return i < sc.n_layers ? i : sc.n_layers - 1;
}

// ----------------------------------------------------------------------------------------
// Depth-profiled layers (alb_sim/physics/models/water.py:85-101,190-245 and
// utils/parameter_profile.py:46-99), evaluated per integration step at the local depth z
// below the layer top (depth - float32 layer offset, water.py:306-308).
// ----------------------------------------------------------------------------------------

// Profile value at local depth z of a layer of height h: kind 1 is LinearParameter
// (float32: t = f32(z / h), f32(start) + t * f32(end - start)), kind 2 ExponentialParameter
// (float64), kind 0 the constant `p0`.
ALB_DEVICE double profile_value(int kind, double p0, double p1, double z, double h) {
    if (kind == 1) {
        const float t = __double2float_rn(z / h);
        return (double)__fadd_rn(__double2float_rn(p0), __fmul_rn(t, __double2float_rn(p1 - p0)));
    }
    if (kind == 2) {
        const double l0 = log(p0), l1 = log(p1);
        return exp(l0 + (z / h) * (l1 - l0));
    }
    return p0;
}

// numpy.interp(f32(z), lut_z, lut_alpha) (clamped at both ends), in float64
ALB_DEVICE double profile_alpha64(const SceneDev& sc, int L, double z) {
    const float* xp = sc.layer_lut_z[L];
    const double* fp = sc.layer_lut_a[L];
    const int n = sc.layer_lut_n[L];
    const double x = (double)__double2float_rn(z);
    if (!(x >= (double)xp[0])) return fp[0];
    if (x >= (double)xp[n - 1]) return fp[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((double)xp[mid] <= x) lo = mid;
        else hi = mid;
    }
    if (x == (double)xp[lo]) return fp[lo];
    const double slope = __ddiv_rn(__dsub_rn(fp[lo + 1], fp[lo]), __dsub_rn((double)xp[lo + 1], (double)xp[lo]));
    return __dadd_rn(__dmul_rn(slope, __dsub_rn(x, (double)xp[lo])), fp[lo]);
}

ALB_DEVICE double local_depth(const SceneDev& sc, int L, double y) { return -(y - sc.ys) - sc.layer_top32[L]; }

// speed of the integration step that starts at height y in water layer L: f32(c / n(z))
ALB_DEVICE double water_speed(const SceneDev& sc, int L, double y) {
    if (!sc.layer_prof[L]) return sc.layer_speed[L];
    const double z = local_depth(sc, L, y);
    const int kind = sc.layer_nkind[L];
    const double n = profile_value(kind, sc.layer_n0[L], sc.layer_n1[L], z, sc.layer_h[L]);
    if (kind == 1) return (double)__fdiv_rn(299800000.0f, (float)n);  // float32 profile
    return (double)__double2float_rn(299800000.0 / n);
}

// attenuation (float32) at height y in water
ALB_DEVICE float water_alpha(const SceneDev& sc, double y) {
    const int L = layer_of(sc, y);
    if (!sc.layer_prof[L]) return sc.layer_alpha[L];
    return __double2float_rn(profile_alpha64(sc, L, local_depth(sc, L, y)));
}

// single-scattering albedo (float32) at height y: (alpha - a) / alpha with the LUT alpha
ALB_DEVICE float water_ssa(const SceneDev& sc, double y) {
    const int L = layer_of(sc, y);
    if (!sc.layer_prof[L]) return sc.layer_ssa[L];
    const double z = local_depth(sc, L, y);
    const double al = profile_alpha64(sc, L, z);
    const double a = profile_value(sc.layer_akind[L], sc.layer_a0[L], sc.layer_a1[L], z, sc.layer_h[L]);
    return __double2float_rn(__ddiv_rn(__dsub_rn(al, a), al));
}

ALB_DEVICE double norm3(double x, double y, double z) {
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
}

// Smallest n >= 1 (<= nmax + 1) with y0 + n * sy <= lim, for sy < 0 and y0 > lim.
ALB_DEVICE int64_t first_at_or_below(double y0, double sy, double lim, int64_t nmax) {
    double est = (lim - y0) / sy;
    if (!(est < (double)nmax + 1.0)) return nmax + 1;
    int64_t n = (int64_t)ceil(est);
    if (n < 1) n = 1;
    while (n > 1 && fma((double)(n - 1), sy, y0) <= lim) --n;
    while (!(fma((double)n, sy, y0) <= lim)) {
        ++n;
        if (n > nmax) return nmax + 1;
    }
    return n;
}

// Smallest n >= 1 (<= nmax + 1) with y0 + n * sy > lim, for sy > 0 and y0 <= lim.
ALB_DEVICE int64_t first_above(double y0, double sy, double lim, int64_t nmax) {
    double est = (lim - y0) / sy;
    if (!(est < (double)nmax + 1.0)) return nmax + 1;
    int64_t n = (int64_t)floor(est) + 1;
    if (n < 1) n = 1;
    while (n > 1 && fma((double)(n - 1), sy, y0) > lim) --n;
    while (!(fma((double)n, sy, y0) > lim)) {
        ++n;
        if (n > nmax) return nmax + 1;
    }
    return n;
}

// Smallest j >= 1 (<= nmax + 1) at which the step start y0 + j * sy lies in a layer other
// than `layer` (multi-layer water only).
ALB_DEVICE int64_t first_layer_change(const SceneDev& sc, int layer, double y0, double sy, int64_t nmax) {
    if (sc.n_layers <= 1 || sy == 0.0) return nmax + 1;
    double lim;
    if (sy < 0.0) {
        if (layer >= sc.n_layers - 1) return nmax + 1;
        lim = sc.ys - sc.layer_bottom[layer];       // deeper than this -> next layer
    } else {
        if (layer == 0) return nmax + 1;
        lim = sc.ys - sc.layer_bottom[layer - 1];   // shallower than this -> previous layer
    }
    double est = (lim - y0) / sy;
    if (!(est < (double)nmax + 1.0)) return nmax + 1;
    int64_t n = (int64_t)floor(est);
    if (n < 1) n = 1;
    while (n > 1 && layer_of(sc, fma((double)(n - 1), sy, y0)) != layer) --n;
    int guard = 0;
    while (layer_of(sc, fma((double)n, sy, y0)) == layer) {
        ++n;
        if (n > nmax || ++guard > 64) return nmax + 1;
    }
    return n;
}

// tau <- fl32(fl64(tau) + inc), at most nmax times; returns the 1-based count of the first
// step with tau >= target (tau then holds that value) or 0 when no step reaches it (tau
// then holds the value after nmax steps). Exact emulation of the reference's float32
// accumulation (core/simulation.py:339-344): within the float32 binade [2^e, 2^e+1) every
// step adds the same rounded increment D, so runs of steps are taken in integer units of
// the binade's ulp and only binade crossings are stepped explicitly.
ALB_DEVICE int64_t tau_run(float& tau, double inc, float target, int64_t nmax) {
    int64_t m = 0;
    int guard = 0;
    while (m < nmax) {
        if (++guard > 4096) break;
        float t1 = __double2float_rn(__dadd_rn((double)tau, inc));
        uint32_t bits = __float_as_uint(tau);
        int ex = (int)((bits >> 23) & 0xffu);
        uint32_t b1 = __float_as_uint(t1);
        int ex1 = (int)((b1 >> 23) & 0xffu);
        if (ex == 0 || ex >= 254 || ex1 != ex) {
            // zero / subnormal start, or the step leaves the binade: explicit step
            tau = t1;
            ++m;
            if (tau >= target) return m;
            continue;
        }
        int64_t T = (int64_t)((bits & 0x7fffffu) | 0x800000u);
        int64_t Dk = (int64_t)((b1 & 0x7fffffu) | 0x800000u) - T;
        if (Dk <= 0) {  // increment below half an ulp: tau never changes again
            tau = t1;
            return 0;
        }
        double inc_u = ldexp(inc, 150 - ex);  // inc in units of this binade's ulp
        double If = floor(inc_u);
        if (inc_u - If == 0.5) {  // exact tie: rounding alternates with parity, step it
            tau = t1;
            ++m;
            if (tau >= target) return m;
            continue;
        }
        int64_t I = (int64_t)If;
        int64_t room = (int64_t)(1 << 24) - 1 - T - I;
        int64_t J = (room >= 0) ? room / Dk + 1 : 1;  // steps keeping the sum in the binade
        // first step reaching the target within the run
        int64_t jt;
        uint32_t tb = __float_as_uint(target);
        int tex = (int)((tb >> 23) & 0xffu);
        if (!(target == target) || tex == 255 || tex - ex > 36) {
            jt = INT64_MAX;  // +inf / NaN / far away
        } else if (target <= tau) {
            jt = 1;
        } else {
            int64_t Tt = (int64_t)((tb & 0x7fffffu) | (tex ? 0x800000u : 0u)) << (tex - ex);
            jt = (Tt - T + Dk - 1) / Dk;
        }
        int64_t jmax = J < nmax - m ? J : nmax - m;
        if (jt <= jmax) {
            tau = (float)ldexp((double)(T + jt * Dk), ex - 150);
            return m + jt;
        }
        tau = (float)ldexp((double)(T + jmax * Dk), ex - 150);
        m += jmax;
    }
    return 0;
}

// numpy.interp(u, cdf, theta) restated: linear interpolation with the reference's slope
// table, left/right clamping (alb_sim/physics/scatter/direction.py:35-36).
// numpy.interp(u, cdf, theta); `interval` receives the table interval of the result (see
// score_scatter_after): 0 below cdf[0], i + 1 for cdf[i] <= u < cdf[i + 1].
ALB_DEVICE double interp_theta(const SceneDev& sc, int layer, double u, int& interval) {
    const double* cdf = sc.layer_cdf[layer];
    const double* th = sc.layer_theta[layer];
    const double* sl = sc.layer_slope[layer];
    const int n = ALB_PHASE_DIVISIONS;
    interval = 0;
    if (u < cdf[0]) return th[0];
    interval = n - 1;
    if (u >= cdf[n - 1]) return th[n - 1];
    int lo = 0, hi = n - 1;  // invariant cdf[lo] <= u < cdf[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid; else hi = mid;
    }
    interval = lo + 1;
    if (u == cdf[lo]) return th[lo];
    return __dadd_rn(__dmul_rn(sl[lo], __dsub_rn(u, cdf[lo])), th[lo]);
}

// Rodrigues rotation of +z onto d, rounded to float32 like rotation_from_z_batch
// (alb_sim/math/rotation_matrix.py:39-102), applied to `l` in float64.
ALB_DEVICE void rotate_from_z(double dx, double dy, double dz, double l0, double l1, double l2,
                              double& ox, double& oy, double& oz) {
    double n = norm3(dx, dy, dz);
    double vx = dx / n, vy = dy / n, vz = dz / n;
    double c = vz;
    double R[9];
    if (fabs(c - 1.0) <= 1.0010000000000001e-05) {
        ox = l0; oy = l1; oz = l2;
        return;
    }
    if (fabs(c + 1.0) <= 1.0010000000000001e-05) {
        ox = l0; oy = -l1; oz = -l2;
        return;
    }
    double ax = -vy, ay = vx;
    double s2 = __dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay));
    double f = (1.0 - c) / s2;
    double axy = __dmul_rn(ay, ax);
    R[0] = __dadd_rn(1.0, __dmul_rn(-__dmul_rn(ay, ay), f));
    R[1] = __dmul_rn(axy, f);
    R[2] = ay;
    R[3] = __dmul_rn(axy, f);
    R[4] = __dadd_rn(1.0, __dmul_rn(-__dmul_rn(ax, ax), f));
    R[5] = -ax;
    R[6] = -ay;
    R[7] = ax;
    R[8] = __dadd_rn(1.0, __dmul_rn(-s2, f));
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = (double)__double2float_rn(R[i]);
    ox = __dadd_rn(__dadd_rn(__dmul_rn(R[0], l0), __dmul_rn(R[1], l1)), __dmul_rn(R[2], l2));
    oy = __dadd_rn(__dadd_rn(__dmul_rn(R[3], l0), __dmul_rn(R[4], l1)), __dmul_rn(R[5], l2));
    oz = __dadd_rn(__dadd_rn(__dmul_rn(R[6], l0), __dmul_rn(R[7], l1)), __dmul_rn(R[8], l2));
}

// Schlick Fresnel, alb_sim/physics/reflection/fresnel.py:14-29
ALB_DEVICE double schlick64(double f0, double cos_i) {
    double x = 1.0 - cos_i;
    double p = pow(x, 5.0);
    return f0 + (1.0 - f0) * p;
}

// ----------------------------------------------------------------------------------------
// Record / query output
// ----------------------------------------------------------------------------------------

template <int PASS>
ALB_DEVICE void emit_event(const TraceOut& out, int channel, int qkind, const Ph& ph,
                           double x, double y, double z, int64_t step, uint32_t pid) {
    float t = __fadd_rn(ph.t0, (float)step);
    if (PASS == ALB_FORWARD) {
        unsigned long long slot = warp_append(out.rec_count, channel);
        if (slot < out.rec_cap[channel]) {
            out.rec_a[channel][2 * slot] = make_float4((float)x, (float)y, (float)z, ph.E);
            out.rec_b[channel][2 * slot] = make_float4((float)ph.dx, (float)ph.dy, (float)ph.dz, t);
            if (out.rec_fwi[channel]) {
                out.rec_fwi[channel][slot] = make_float4(ph.fwi[0], ph.fwi[1], ph.fwi[2], 0.f);
                out.rec_sfi[channel][slot] = make_float4(ph.sfi[0], ph.sfi[1], ph.sfi[2], 0.f);
            }
            if (out.rec_id[channel]) out.rec_id[channel][slot] = pid;
            if (out.rec_sco[channel]) out.rec_sco[channel][slot] = make_float4(ph.sc.a, ph.sc.b, ph.sc.g, ph.sc.l);
        }
    } else {
        unsigned long long slot = warp_append(out.q_count, qkind);
        if (slot < out.q_cap[qkind]) {
            if (out.q_s[qkind]) out.q_s[qkind][slot] = make_float4(ph.sc.a, ph.sc.b, ph.sc.g, ph.sc.l);
            float xh = (float)x, yh = (float)y, zh = (float)z;
            out.q_a[qkind][slot] = make_float4(xh, yh, zh, ph.E);
            out.q_b[qkind][slot] = make_float4((float)ph.dx, (float)ph.dy, (float)ph.dz, t);
            out.q_c[qkind][slot] = make_float4((float)(x - (double)xh), (float)(y - (double)yh),
                                               (float)(z - (double)zh), 0.f);
            if (out.q_id[qkind]) out.q_id[qkind][slot] = pid;
        }
    }
}

// ----------------------------------------------------------------------------------------
// Event handlers (one crossing step each)
// ----------------------------------------------------------------------------------------

// Extension (no counterpart in the reference, whose surface normal is +y / -y): Gaussian
// surface slopes. At every surface interaction the facet normal is normalize(-gx, 1, -gz)
// with slope components gx, gz ~ N(0, sigma^2) (one Box-Muller block). Reflection, Snell
// refraction and the Fresnel factor use the facet; a facet facing away from the photon, or
// one that would send it to the wrong side of the mean surface, falls back to the flat one.
template <class Src>
ALB_DEVICE void draw_facet(const SceneDev& sc, Src& src, double& mx, double& my, double& mz) {
    double n0, n1, n2;
    draw_normals(src, n0, n1, n2);
    const double gx = n0 * sc.slope_sigma, gz = n1 * sc.slope_sigma;
    const double nn = norm3(gx, 1.0, gz);
    mx = -gx / nn;
    my = 1.0 / nn;
    mz = -gz / nn;
}

template <int PASS, class Src>
ALB_DEVICE void handle_enter(const SceneDev& sc, const TraceOut& out, Ph& ph, Src& src,
                             double svx, double svy, double svz, uint32_t pid) {
    double nx = ph.px + svx, ny = ph.py + svy, nz = ph.pz + svz;
    double stx = nx - ph.px, sty = ny - ph.py, stz = nz - ph.pz;
    double f = (sc.ys - ph.py) / sty;
    f = fmin(fmax(f, 0.0), 1.0);
    double xs = ph.px + f * stx, ys = ph.py + f * sty, zs = ph.pz + f * stz;
    ph.fwi[0] = (float)xs; ph.fwi[1] = (float)ys; ph.fwi[2] = (float)zs;
    double F = schlick64(sc.f0, -ph.dy);
    emit_event<PASS>(out, ALB_SURFACE_REFLECTION, kQuerySurface, ph, xs, ys, zs, ph.s, pid);
    double eta = sc.eta;
    bool flat = true;
    if (sc.slope_sigma > 0.0) {
        double mx, my, mz;
        draw_facet(sc, src, mx, my, mz);
        double ci = -(ph.dx * mx + ph.dy * my + ph.dz * mz);
        if (ci > 0.0) {
            ci = fmin(ci, 1.0);
            double ct = sqrt(fmax(0.0, 1.0 - (eta * eta) * (1.0 - ci * ci)));
            double k = eta * ci - ct;
            double tx = eta * ph.dx + k * mx, ty = eta * ph.dy + k * my, tz = eta * ph.dz + k * mz;
            if (ty < 0.0) {
                double tn = norm3(tx, ty, tz);
                ph.dx = tx / tn; ph.dy = ty / tn; ph.dz = tz / tn;
                F = schlick64(sc.f0, ci);
                flat = false;
            }
        }
    }
    if (flat) {
        // Snell, air -> water, normal +y
        double ci = fmin(fmax(-ph.dy, -1.0), 1.0);
        double sin2 = (eta * eta) * (1.0 - ci * ci);
        double ct = sqrt(fmax(0.0, 1.0 - sin2));
        double tx = eta * ph.dx, ty = eta * ph.dy + (eta * ci - ct), tz = eta * ph.dz;
        double tn = norm3(tx, ty, tz);
        ph.dx = tx / tn; ph.dy = ty / tn; ph.dz = tz / tn;
    }
    ph.E = (float)((double)ph.E * (1.0 - F));
    double len = norm3(stx, sty, stz);
    double rem = (1.0 - f) * len;
    ph.px = xs + ph.dx * rem; ph.py = ys + ph.dy * rem; ph.pz = zs + ph.dz * rem;
    ph.taut = draw_tau(src);
}

template <int PASS, class Src>
ALB_DEVICE void handle_exit(const SceneDev& sc, const TraceOut& out, Ph& ph, Src& src,
                            double svx, double svy, double svz, uint32_t pid) {
    double nx = ph.px + svx, ny = ph.py + svy, nz = ph.pz + svz;
    double stx = nx - ph.px, sty = ny - ph.py, stz = nz - ph.pz;
    double f = (sc.ys - ph.py) / sty;
    f = fmin(fmax(f, 0.0), 1.0);
    double xs = ph.px + f * stx, ys = ph.py + f * sty, zs = ph.pz + f * stz;
    double mx = 0.0, my = 1.0, mz = 0.0, cf = ph.dy;  // facet (upward) and cos to it
    bool tilted = false;
    if (sc.slope_sigma > 0.0) {
        draw_facet(sc, src, mx, my, mz);
        cf = ph.dx * mx + ph.dy * my + ph.dz * mz;
        tilted = cf > 0.0;
        if (!tilted) { mx = 0.0; my = 1.0; mz = 0.0; cf = ph.dy; }
    }
    double F = schlick64(sc.f0, tilted ? fmin(cf, 1.0) : ph.dy);
    double U = draw_uniform(src);
    bool reflect = U < F;
    if (PASS == ALB_FORWARD && !reflect)
        emit_event<PASS>(out, ALB_SURFACE_TRANSMISSION_UP, 0, ph, xs, ys, zs, ph.s, pid);
    // Snell with the reference's fixed 1 -> n_water ratio and normal -y
    double eta = sc.eta;
    double ci = fmin(fmax(tilted ? cf : ph.dy, -1.0), 1.0);
    double sin2 = (eta * eta) * (1.0 - ci * ci);
    double ct = sqrt(fmax(0.0, 1.0 - sin2));
    reflect = reflect || (sin2 > 1.0);
    double len = norm3(stx, sty, stz);
    bool done = false;
    if (tilted) {
        if (reflect) {
            double rx = ph.dx - 2.0 * cf * mx, ry = ph.dy - 2.0 * cf * my, rz = ph.dz - 2.0 * cf * mz;
            if (ry < 0.0) {
                ph.dx = rx; ph.dy = ry; ph.dz = rz;
                done = true;
            }
        } else {
            double k = eta * ci - ct;
            double tx = eta * ph.dx - k * mx, ty = eta * ph.dy - k * my, tz = eta * ph.dz - k * mz;
            if (ty > 0.0) {
                double tn = norm3(tx, ty, tz);
                ph.dx = tx / tn; ph.dy = ty / tn; ph.dz = tz / tn;
                done = true;
            }
        }
    }
    if (!done) {
        if (reflect) {
            ph.dy = -ph.dy;
        } else {
            double cf0 = fmin(fmax(ph.dy, -1.0), 1.0);
            double ct0 = sqrt(fmax(0.0, 1.0 - (eta * eta) * (1.0 - cf0 * cf0)));
            double tx = eta * ph.dx, ty = eta * ph.dy - (eta * cf0 - ct0), tz = eta * ph.dz;
            double tn = norm3(tx, ty, tz);
            ph.dx = tx / tn; ph.dy = ty / tn; ph.dz = tz / tn;
        }
    }
    double rem = (1.0 - f) * len;
    ph.px = xs + ph.dx * rem; ph.py = ys + ph.dy * rem; ph.pz = zs + ph.dz * rem;
    if (reflect) {
        float a = water_alpha(sc, ph.py);
        if (sc.adjoint) score_tau(sc, ph.sc, layer_of(sc, ph.py), (float)((double)a * len));
        ph.tau = __double2float_rn(__dadd_rn((double)ph.tau, (double)a * len));
    }
}

template <int PASS, class Src>
ALB_DEVICE void handle_floor(const SceneDev& sc, const TraceOut& out, Ph& ph, Src& src,
                             double svx, double svy, double svz, uint32_t pid) {
    double nx = ph.px + svx, ny = ph.py + svy, nz = ph.pz + svz;
    double stx = nx - ph.px, sty = ny - ph.py, stz = nz - ph.pz;
    double f = (sc.yf - ph.py) / sty;
    f = fmin(fmax(f, 0.0), 1.0);
    double xb = ph.px + f * stx, yb = ph.py + f * sty, zb = ph.pz + f * stz;
    ph.sfi[0] = (float)xb; ph.sfi[1] = (float)yb; ph.sfi[2] = (float)zb;
    if (PASS == ALB_FORWARD && out.hm_radius && ph.fwi[0] == ph.fwi[0]) {
        // accumulate_scatter_radius_heatmap (alb_sim/math/accumulate_heatmap.py:64-124)
        double ax = (double)ph.fwi[0] - sc.wc[0], az = (double)ph.fwi[2] - sc.wc[2];
        double bx = xb - sc.fc[0], bz = zb - sc.fc[2];
        double rs = sqrt(ax * ax + az * az), rf = sqrt(bx * bx + bz * bz);
        long long xi = (long long)((rs / sc.hm_wext) * sc.hm_bins);
        long long yi = (long long)((rf / sc.hm_fext) * sc.hm_bins);
        if (xi >= 0 && xi < sc.hm_bins && yi >= 0 && yi < sc.hm_bins)
            atomicAdd(out.hm_radius + xi * sc.hm_bins + yi, 1u);
    }
    emit_event<PASS>(out, ALB_BOTTOM_REFLECTION, kQueryBottom, ph, xb, yb, zb, ph.s, pid);
    double n0, n1, n2;
    draw_normals(src, n0, n1, n2);
    float g0 = (float)n0, g1 = (float)n1, g2 = (float)n2;
    float gn = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(g0, g0), __fmul_rn(g1, g1)), __fmul_rn(g2, g2)));
    g0 = __fdiv_rn(g0, gn); g1 = __fdiv_rn(g1, gn); g2 = __fdiv_rn(g2, gn);
    double hx = (double)g0, hy = 1.0 + (double)g1, hz = (double)g2;
    double hn = norm3(hx, hy, hz);
    ph.dx = hx / hn; ph.dy = hy / hn; ph.dz = hz / hn;
    double len = norm3(stx, sty, stz);
    double rem = (1.0 - f) * len;
    ph.px = xb + ph.dx * rem; ph.py = yb + ph.dy * rem; ph.pz = zb + ph.dz * rem;
    float a = water_alpha(sc, ph.py);
    if (sc.adjoint) {
        score_tau(sc, ph.sc, layer_of(sc, ph.py), (float)((double)a * len));
        ph.sc.l += sc.inv_albedo;
    }
    ph.tau = __double2float_rn(__dadd_rn((double)ph.tau, (double)a * len));
    ph.E = __fmul_rn(ph.E, sc.floor_albedo32);
}

template <int PASS, class Src>
ALB_DEVICE void handle_scatter(const SceneDev& sc, const TraceOut& out, Ph& ph, Src& src,
                               int64_t step, uint32_t pid) {
    int L = layer_of(sc, ph.py);
    if (sc.adjoint) score_scatter_density(sc, ph.sc, L);
    emit_event<PASS>(out, ALB_SCATTER, kQueryScatter, ph, ph.px, ph.py, ph.pz, step, pid);
    double uth, phi;
    float new_target;
    draw_scatter(src, uth, phi, new_target);
    int interval;
    double th = interp_theta(sc, L, uth, interval);
    double st, ct, sp, cp;
    sincos(th, &st, &ct);
    sincos(phi, &sp, &cp);
    double l0 = st * cp, l1 = st * sp, l2 = ct;
    double ox, oy, oz;
    rotate_from_z(ph.dx, ph.dy, ph.dz, l0, l1, l2, ox, oy, oz);
    ph.dx = ox; ph.dy = oy; ph.dz = oz;
    if (sc.adjoint) score_scatter_after(sc, ph.sc, L, (float)ct, interval);
    ph.E = __fmul_rn(ph.E, water_ssa(sc, ph.py));
    ph.tau = __fsub_rn(ph.tau, ph.taut);
    ph.taut = new_target;
}

// ----------------------------------------------------------------------------------------
// Emission (alb_sim/physics/models/simulation.py:130-208)
// ----------------------------------------------------------------------------------------

template <int PASS, class Src>
ALB_DEVICE void emit_photon(const SceneDev& sc, Ph& ph, Src& src) {
    const double* R = sc.rot_d;
    ph.px = 0.0; ph.py = 0.0; ph.pz = 0.0;
    ph.E = 1.0f; ph.tau = 0.0f; ph.taut = __int_as_float(0x7f800000); ph.s = 0;
    ph.sc = Score{0.f, 0.f, 0.f, 0.f};
    float qnan = __int_as_float(0x7fc00000);
    ph.fwi[0] = ph.fwi[1] = ph.fwi[2] = qnan;
    ph.sfi[0] = ph.sfi[1] = ph.sfi[2] = qnan;
    if (PASS == ALB_FORWARD) {
        double th, phi, pulse;
        draw_emit_fwd(sc, src, th, phi, pulse);
        double st = sin(th), ct = cos(th);
        double l0 = st * cos(phi), l1 = st * sin(phi), l2 = ct;
        ph.dx = (double)(float)__dadd_rn(__dadd_rn(__dmul_rn(l0, R[0]), __dmul_rn(l1, R[1])), __dmul_rn(l2, R[2]));
        ph.dy = (double)(float)__dadd_rn(__dadd_rn(__dmul_rn(l0, R[3]), __dmul_rn(l1, R[4])), __dmul_rn(l2, R[5]));
        ph.dz = (double)(float)__dadd_rn(__dadd_rn(__dmul_rn(l0, R[6]), __dmul_rn(l1, R[7])), __dmul_rn(l2, R[8]));
        ph.t0 = __fdiv_rn((float)pulse, (float)sc.eff_rate32);
    } else {
        double x1, x2, z, phc;
        draw_emit_bwd(sc, src, x1, x2, z, phc);
        double r = sc.aperture * sqrt(x1);
        double a = kTwoPi * x2;
        double d0 = r * cos(a), d1 = r * sin(a);
        double ox = __dadd_rn(__dadd_rn(__dmul_rn(d0, R[0]), __dmul_rn(d1, R[1])), __dmul_rn(0.0, R[2]));
        double oy = __dadd_rn(__dadd_rn(__dmul_rn(d0, R[3]), __dmul_rn(d1, R[4])), __dmul_rn(0.0, R[5]));
        double oz = __dadd_rn(__dadd_rn(__dmul_rn(d0, R[6]), __dmul_rn(d1, R[7])), __dmul_rn(0.0, R[8]));
        double st = sqrt(1.0 - z * z);
        double l0 = st * cos(phc), l1 = st * sin(phc), l2 = z;
        float cx = (float)__dadd_rn(__dadd_rn(__dmul_rn(l0, R[0]), __dmul_rn(l1, R[1])), __dmul_rn(l2, R[2]));
        float cy = (float)__dadd_rn(__dadd_rn(__dmul_rn(l0, R[3]), __dmul_rn(l1, R[4])), __dmul_rn(l2, R[5]));
        float cz = (float)__dadd_rn(__dadd_rn(__dmul_rn(l0, R[6]), __dmul_rn(l1, R[7])), __dmul_rn(l2, R[8]));
        // the reference adds the aperture point to the DIRECTION (positions start at 0)
        ph.dx = ox + (double)cx; ph.dy = oy + (double)cy; ph.dz = oz + (double)cz;
        ph.t0 = 0.0f;
    }
}

// ----------------------------------------------------------------------------------------
// Full photon
// ----------------------------------------------------------------------------------------

template <int PASS, class Src>
ALB_DEVICE void trace_photon(const SceneDev& sc, const TraceOut& out, Ph& ph, Src& src, uint32_t pid,
                             unsigned long long& events) {
    const int64_t S = sc.stop_step[PASS];
    int guard = 0;
    while (ph.s < S) {
        if (++guard > kMaxEventsPerPhoton) {
            set_err(out.err, ALB_ERR_ITER_CAP);
            break;
        }
        const int64_t left = S - ph.s;
        if (ph.py > sc.ys) {
            // in air: nothing happens until the step that crosses the surface
            double v = sc.v_air;
            double svx = (ph.dx * v) * sc.dt, svy = (ph.dy * v) * sc.dt, svz = (ph.dz * v) * sc.dt;
            int64_t n = (svy < 0.0) ? first_at_or_below(ph.py, svy, sc.ys, left) : left + 1;
            if (n - 1 >= left) {
                double k = (double)left;
                ph.px = fma(k, svx, ph.px); ph.py = fma(k, svy, ph.py); ph.pz = fma(k, svz, ph.pz);
                ph.s = S;
                break;
            }
            double k = (double)(n - 1);
            ph.px = fma(k, svx, ph.px); ph.py = fma(k, svy, ph.py); ph.pz = fma(k, svz, ph.pz);
            ph.s += n - 1;
            handle_enter<PASS>(sc, out, ph, src, svx, svy, svz, pid);
            ph.s += 1;
            ++events;
        } else if (sc.layer_prof[layer_of(sc, ph.py)]) {
            // depth-profiled layer: one integration step, speed and attenuation at its start
            --guard;  // bounded by the step count, not an event
            const int L = layer_of(sc, ph.py);
            const double v = water_speed(sc, L, ph.py);
            const double svx = (ph.dx * v) * sc.dt, svy = (ph.dy * v) * sc.dt, svz = (ph.dz * v) * sc.dt;
            const double ny = ph.py + svy;
            if (ny > sc.ys) {
                handle_exit<PASS>(sc, out, ph, src, svx, svy, svz, pid);
                ph.s += 1;
                ++events;
                ++guard;
                continue;
            }
            if (ny <= sc.yf) {
                handle_floor<PASS>(sc, out, ph, src, svx, svy, svz, pid);
                ph.s += 1;
                ++events;
                ++guard;
                continue;
            }
            const double len = norm3(svx, svy, svz);
            const float a = __double2float_rn(profile_alpha64(sc, L, local_depth(sc, L, ph.py)));
            ph.tau = __double2float_rn(__dadd_rn((double)ph.tau, (double)a * len));
            ph.px = ph.px + svx;
            ph.py = ny;
            ph.pz = ph.pz + svz;
            const int64_t step = ph.s;
            ph.s += 1;
            if (ph.tau >= ph.taut) {
                handle_scatter<PASS>(sc, out, ph, src, step, pid);
                ++events;
                ++guard;
            }
        } else {
            int L = layer_of(sc, ph.py);
            double v = sc.layer_speed[L];
            double svx = (ph.dx * v) * sc.dt, svy = (ph.dy * v) * sc.dt, svz = (ph.dz * v) * sc.dt;
            double len = norm3(svx, svy, svz);
            int64_t n_plane = left + 1;
            if (svy > 0.0) n_plane = first_above(ph.py, svy, sc.ys, left) - 1;
            else if (svy < 0.0) n_plane = first_at_or_below(ph.py, svy, sc.yf, left) - 1;
            int64_t n_layer = first_layer_change(sc, L, ph.py, svy, left);
            int64_t nseg = n_plane < n_layer ? n_plane : n_layer;
            if (nseg > left) nseg = left;
            double inc = (double)sc.layer_alpha[L] * len;
            int64_t m = (nseg > 0) ? tau_run(ph.tau, inc, ph.taut, nseg) : 0;
            // optical depth of the run: m steps to the scatter, else the whole segment
            if (sc.adjoint) score_tau(sc, ph.sc, L, (float)((double)(m > 0 ? m : nseg) * inc));
            if (m > 0) {
                double k = (double)m;
                ph.px = fma(k, svx, ph.px); ph.py = fma(k, svy, ph.py); ph.pz = fma(k, svz, ph.pz);
                int64_t step = ph.s + m - 1;
                handle_scatter<PASS>(sc, out, ph, src, step, pid);
                ph.s = step + 1;
                ++events;
                continue;
            }
            double k = (double)nseg;
            ph.px = fma(k, svx, ph.px); ph.py = fma(k, svy, ph.py); ph.pz = fma(k, svz, ph.pz);
            ph.s += nseg;
            if (ph.s >= S) break;
            if (nseg == n_plane) {
                if (svy > 0.0) handle_exit<PASS>(sc, out, ph, src, svx, svy, svz, pid);
                else handle_floor<PASS>(sc, out, ph, src, svx, svy, svz, pid);
                ph.s += 1;
                ++events;
            }
        }
    }
}

}  // namespace alb
