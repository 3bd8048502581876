// Fast tracer: float32 event-jump form of the reference's integrator for Philox streams.
//
// Same physics and the same event sequence as tracer.cuh (alb_sim/core/simulation.py:
// 220-570), restated for throughput: positions, directions and the optical-depth run are
// float32, the number of steps to the next scatter is the closed form
// ceil((tau* - tau) / (alpha |step|)), the scattering angle comes from a 65 537-entry
// inverse-CDF table of the reference's phase-function table, and directions are rotated
// in an orthonormal frame built from the incoming direction (Duff et al. 2017, "Building an
// orthonormal basis, revisited"). The variates are drawn in the same distributions as the
// reference (uniforms, truncated Rayleigh, isotropic unit vectors), so the result agrees
// with the reference in distribution; replay-exact runs use the precise tracer.
#pragma once

#include "device_common.cuh"
#include "tracer.cuh"

namespace alb {

constexpr int kInvCdf = 65536;  // inverse-CDF table has kInvCdf + 1 entries per layer

struct FastScene {
    const float* inv_theta[ALB_MAX_LAYERS];  // theta(u) at u = j / kInvCdf
};

struct PhF {
    float px, py, pz;
    float dx, dy, dz;
    float E, tau, taut, t0;
    float fwi[3], sfi[3];
    int s;
    Score sc;  // adjoint path score (see score_tau in tracer.cuh)
};

// (x / 2^9 + 0.5) / 2^23: an exact float strictly inside (0, 1), 2^23 equally spaced values
ALB_DEVICE float uf(uint32_t x) { return ((float)(x >> 9) + 0.5f) * 1.1920928955078125e-07f; }

ALB_DEVICE int layer_of_f(const SceneDev& sc, float y) {
    float depth = -(y - (float)sc.ys);
    int i = 0;
    while (i < sc.n_layers && !((float)sc.layer_bottom[i] > depth)) ++i;
    return i < sc.n_layers ? i : sc.n_layers - 1;
}

template <int PASS>
ALB_DEVICE void emit_event_f(const TraceOut& out, int channel, int qkind, const PhF& ph, float x, float y, float z,
                             int step, uint32_t pid) {
    float t = __fadd_rn(ph.t0, (float)step);
    if (PASS == ALB_FORWARD) {
        unsigned long long slot = warp_append(out.rec_count, channel);
        if (slot < out.rec_cap[channel]) {
            out.rec_a[channel][2 * slot] = make_float4(x, y, z, ph.E);
            out.rec_b[channel][2 * slot] = make_float4(ph.dx, ph.dy, ph.dz, t);
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
            out.q_a[qkind][slot] = make_float4(x, y, z, ph.E);
            out.q_b[qkind][slot] = make_float4(ph.dx, ph.dy, ph.dz, t);
            out.q_c[qkind][slot] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (out.q_id[qkind]) out.q_id[qkind][slot] = pid;
        }
    }
}

ALB_DEVICE float schlick_f(float f0, float c) {
    float x = 1.f - c;
    float x2 = x * x;
    return f0 + (1.f - f0) * (x2 * x2 * x);
}

// first n >= 1 with y0 + n*sy <= lim (sy < 0, y0 > lim), clamped to nmax + 1
ALB_DEVICE int first_at_or_below_f(float y0, float sy, float lim, int nmax) {
    float est = (lim - y0) / sy;
    if (!(est < (float)nmax + 1.f)) return nmax + 1;
    int n = (int)ceilf(est);
    return n < 1 ? 1 : n;
}
// first n >= 1 with y0 + n*sy > lim (sy > 0, y0 <= lim)
ALB_DEVICE int first_above_f(float y0, float sy, float lim, int nmax) {
    float est = (lim - y0) / sy;
    if (!(est < (float)nmax + 1.f)) return nmax + 1;
    int n = (int)floorf(est) + 1;
    return n < 1 ? 1 : n;
}

ALB_DEVICE int first_layer_change_f(const SceneDev& sc, int layer, float y0, float sy, int nmax) {
    if (sc.n_layers <= 1 || sy == 0.f) return nmax + 1;
    float lim;
    if (sy < 0.f) {
        if (layer >= sc.n_layers - 1) return nmax + 1;
        lim = (float)(sc.ys - sc.layer_bottom[layer]);
        int n = first_at_or_below_f(y0, sy, lim, nmax);
        return n;
    }
    if (layer == 0) return nmax + 1;
    lim = (float)(sc.ys - sc.layer_bottom[layer - 1]);
    return first_above_f(y0, sy, lim, nmax);
}

// attenuation at height y (float32 layer lookup; profiled layers through the exact table)
ALB_DEVICE float water_alpha_f(const SceneDev& sc, float y) {
    const int L = layer_of_f(sc, y);
    return sc.layer_prof[L] ? water_alpha(sc, (double)y) : sc.layer_alpha[L];
}

// Gaussian surface slopes (extension; see draw_facet in tracer.cuh): facet normal
// normalize(-gx, 1, -gz), gx, gz ~ N(0, sigma^2) from one Box-Muller block.
ALB_DEVICE void draw_facet_f(const SceneDev& sc, PhiloxSrc& src, float& mx, float& my, float& mz) {
    U4 b = src.block();
    const float r = sqrtf(-2.f * __logf(uf(b.x)));
    float sa, ca;
    __sincosf(6.283185307179586f * uf(b.y), &sa, &ca);
    const float s = (float)sc.slope_sigma;
    const float gx = r * ca * s, gz = r * sa * s;
    const float inv = rsqrtf(fmaf(gx, gx, fmaf(gz, gz, 1.f)));
    mx = -gx * inv;
    my = inv;
    mz = -gz * inv;
}

template <int PASS>
ALB_DEVICE void trace_photon_fast(const SceneDev& sc, const FastScene& fs, const TraceOut& out, PhF& ph,
                                  PhiloxSrc& src, uint32_t pid, unsigned long long& events) {
    const int S = (int)sc.stop_step[PASS];
    const float ys = (float)sc.ys, yf = (float)sc.yf, dt = (float)sc.dt;
    const float eta = (float)sc.eta, f0 = (float)sc.f0;
    int guard = 0;
    while (ph.s < S) {
        if (++guard > kMaxEventsPerPhoton) {
            set_err(out.err, ALB_ERR_ITER_CAP);
            break;
        }
        const int left = S - ph.s;
        if (ph.py > ys) {
            float v = (float)sc.v_air * dt;
            float svx = ph.dx * v, svy = ph.dy * v, svz = ph.dz * v;
            int n = (svy < 0.f) ? first_at_or_below_f(ph.py, svy, ys, left) : left + 1;
            if (n - 1 >= left) {
                float k = (float)left;
                ph.px = fmaf(k, svx, ph.px); ph.py = fmaf(k, svy, ph.py); ph.pz = fmaf(k, svz, ph.pz);
                ph.s = S;
                break;
            }
            float k = (float)(n - 1);
            ph.px = fmaf(k, svx, ph.px); ph.py = fmaf(k, svy, ph.py); ph.pz = fmaf(k, svz, ph.pz);
            ph.s += n - 1;
            // entering step (handle_enter)
            float f = fminf(fmaxf((ys - ph.py) / svy, 0.f), 1.f);
            float xs = fmaf(f, svx, ph.px), yss = ys, zs = fmaf(f, svz, ph.pz);
            ph.fwi[0] = xs; ph.fwi[1] = yss; ph.fwi[2] = zs;
            float F = schlick_f(f0, -ph.dy);
            emit_event_f<PASS>(out, ALB_SURFACE_REFLECTION, kQuerySurface, ph, xs, yss, zs, ph.s, pid);
            float mx = 0.f, my = 1.f, mz = 0.f;
            if (sc.slope_sigma > 0.0) {
                draw_facet_f(sc, src, mx, my, mz);
                if (!(-(ph.dx * mx + ph.dy * my + ph.dz * mz) > 0.f)) { mx = 0.f; my = 1.f; mz = 0.f; }
            }
            float ci = fminf(fmaxf(-(ph.dx * mx + ph.dy * my + ph.dz * mz), -1.f), 1.f);
            float ct = sqrtf(fmaxf(0.f, 1.f - eta * eta * (1.f - ci * ci)));
            float kt = eta * ci - ct;
            float tx = fmaf(kt, mx, eta * ph.dx), ty = fmaf(kt, my, eta * ph.dy), tz = fmaf(kt, mz, eta * ph.dz);
            if (!(ty < 0.f)) {  // a steep facet would send the photon up: the mean surface instead
                ci = fminf(fmaxf(-ph.dy, -1.f), 1.f);
                ct = sqrtf(fmaxf(0.f, 1.f - eta * eta * (1.f - ci * ci)));
                tx = eta * ph.dx; ty = eta * ph.dy + (eta * ci - ct); tz = eta * ph.dz;
            }
            F = schlick_f(f0, ci);
            float tn = rsqrtf(fmaf(tx, tx, fmaf(ty, ty, tz * tz)));
            ph.dx = tx * tn; ph.dy = ty * tn; ph.dz = tz * tn;
            ph.E *= (1.f - F);
            float rem = (1.f - f) * sqrtf(fmaf(svx, svx, fmaf(svy, svy, svz * svz)));
            ph.px = fmaf(ph.dx, rem, xs); ph.py = fmaf(ph.dy, rem, yss); ph.pz = fmaf(ph.dz, rem, zs);
            ph.taut = -__logf(uf(src.block().x));
            ph.s += 1;
            ++events;
            continue;
        }
        int L = layer_of_f(sc, ph.py);
        // a depth-profiled layer is crossed one integration step at a time (speed and
        // attenuation at the step's start depth); those steps are not events for the cap
        const bool prof = sc.layer_prof[L] != 0;
        if (prof) --guard;
        float v = (prof ? (float)water_speed(sc, L, (double)ph.py) : (float)sc.layer_speed[L]) * dt;
        float svx = ph.dx * v, svy = ph.dy * v, svz = ph.dz * v;
        float len = sqrtf(fmaf(svx, svx, fmaf(svy, svy, svz * svz)));
        int n_plane = left + 1;
        if (svy > 0.f) n_plane = first_above_f(ph.py, svy, ys, left) - 1;
        else if (svy < 0.f) n_plane = first_at_or_below_f(ph.py, svy, yf, left) - 1;
        int n_layer = prof ? 1 : first_layer_change_f(sc, L, ph.py, svy, left);
        int nseg = min(min(n_plane, n_layer), left);
        float inc = (prof ? water_alpha(sc, (double)ph.py) : sc.layer_alpha[L]) * len;
        int m = 0;
        if (nseg > 0 && inc > 0.f) {
            float need = (ph.taut - ph.tau) / inc;
            m = need <= 1.f ? 1 : (need < (float)nseg + 1.f ? (int)ceilf(need) : nseg + 1);
        } else if (nseg > 0 && ph.tau >= ph.taut) {
            m = 1;
        }
        if (m >= 1 && m <= nseg) {
            float k = (float)m;
            ph.px = fmaf(k, svx, ph.px); ph.py = fmaf(k, svy, ph.py); ph.pz = fmaf(k, svz, ph.pz);
            ph.tau = fmaf(k, inc, ph.tau);
            int step = ph.s + m - 1;
            int L2 = layer_of_f(sc, ph.py);
            if (sc.adjoint) {
                score_tau(sc, ph.sc, L, k * inc);
                score_scatter_density(sc, ph.sc, L2);
            }
            emit_event_f<PASS>(out, ALB_SCATTER, kQueryScatter, ph, ph.px, ph.py, ph.pz, step, pid);
            U4 b = src.block();
            float u = uf(b.x) * (float)kInvCdf;
            int j = min((int)u, kInvCdf - 1);
            const float* tab = fs.inv_theta[L2];
            float th = fmaf(u - (float)j, __ldg(tab + j + 1) - __ldg(tab + j), __ldg(tab + j));
            float st, ctt, sp, cp;
            __sincosf(th, &st, &ctt);
            __sincosf(6.283185307179586f * uf(b.y), &sp, &cp);
            // orthonormal frame around d
            float sg = copysignf(1.f, ph.dz);
            float a = -1.f / (sg + ph.dz);
            float bb = ph.dx * ph.dy * a;
            float t1x = 1.f + sg * ph.dx * ph.dx * a, t1y = sg * bb, t1z = -sg * ph.dx;
            float t2x = bb, t2y = sg + ph.dy * ph.dy * a, t2z = -ph.dy;
            float ux = cp * t1x + sp * t2x, uy = cp * t1y + sp * t2y, uz = cp * t1z + sp * t2z;
            ph.dx = fmaf(ctt, ph.dx, st * ux);
            ph.dy = fmaf(ctt, ph.dy, st * uy);
            ph.dz = fmaf(ctt, ph.dz, st * uz);
            if (sc.adjoint) score_scatter_after(sc, ph.sc, L2, ctt, sample_interval_of_angle(sc, L2, th));
            ph.E *= sc.layer_prof[L2] ? water_ssa(sc, (double)ph.py) : sc.layer_ssa[L2];
            ph.tau = fmaxf(ph.tau - ph.taut, 0.f);
            ph.taut = -__logf(uf(b.z));
            ph.s = step + 1;
            ++events;
            if (prof) ++guard;
            continue;
        }
        float k = (float)nseg;
        ph.px = fmaf(k, svx, ph.px); ph.py = fmaf(k, svy, ph.py); ph.pz = fmaf(k, svz, ph.pz);
        ph.tau = fmaf(k, inc, ph.tau);
        if (sc.adjoint && nseg > 0) score_tau(sc, ph.sc, L, k * inc);
        ph.s += nseg;
        if (ph.s >= S) break;
        if (nseg != n_plane) continue;  // layer change (or one profiled step) only
        if (prof) ++guard;
        if (svy > 0.f) {
            // handle_exit
            float f = fminf(fmaxf((ys - ph.py) / svy, 0.f), 1.f);
            float xs = fmaf(f, svx, ph.px), yss = ys, zs = fmaf(f, svz, ph.pz);
            float mx = 0.f, my = 1.f, mz = 0.f;
            if (sc.slope_sigma > 0.0) {
                draw_facet_f(sc, src, mx, my, mz);
                if (!(ph.dx * mx + ph.dy * my + ph.dz * mz > 0.f)) { mx = 0.f; my = 1.f; mz = 0.f; }
            }
            const float cf = fminf(ph.dx * mx + ph.dy * my + ph.dz * mz, 1.f);
            float F = schlick_f(f0, cf);
            bool reflect = uf(src.block().x) < F;
            if (PASS == ALB_FORWARD && !reflect)
                emit_event_f<PASS>(out, ALB_SURFACE_TRANSMISSION_UP, 0, ph, xs, yss, zs, ph.s, pid);
            if (reflect) {
                const float rx = ph.dx - 2.f * cf * mx, ry = ph.dy - 2.f * cf * my, rz = ph.dz - 2.f * cf * mz;
                if (ry < 0.f) { ph.dx = rx; ph.dy = ry; ph.dz = rz; }
                else ph.dy = -ph.dy;
            } else {
                float ci = fmaxf(cf, -1.f);
                float ct = sqrtf(fmaxf(0.f, 1.f - eta * eta * (1.f - ci * ci)));
                float k = eta * ci - ct;
                float tx = fmaf(-k, mx, eta * ph.dx), ty = fmaf(-k, my, eta * ph.dy), tz = fmaf(-k, mz, eta * ph.dz);
                if (!(ty > 0.f)) {
                    ci = fminf(fmaxf(ph.dy, -1.f), 1.f);
                    ct = sqrtf(fmaxf(0.f, 1.f - eta * eta * (1.f - ci * ci)));
                    tx = eta * ph.dx; ty = eta * ph.dy - (eta * ci - ct); tz = eta * ph.dz;
                }
                float tn = rsqrtf(fmaf(tx, tx, fmaf(ty, ty, tz * tz)));
                ph.dx = tx * tn; ph.dy = ty * tn; ph.dz = tz * tn;
            }
            float rem = (1.f - f) * len;
            ph.px = fmaf(ph.dx, rem, xs); ph.py = fmaf(ph.dy, rem, yss); ph.pz = fmaf(ph.dz, rem, zs);
            if (reflect) {
                const float a = water_alpha_f(sc, ph.py);
                if (sc.adjoint) score_tau(sc, ph.sc, layer_of_f(sc, ph.py), a * len);
                ph.tau = fmaf(a, len, ph.tau);
            } else if (!(ph.py > ys)) {
                // A transmitted photon is in the air. Near the surface a float32 height is
                // quantised to ulp(ys) (3e-5 m at 400 m), as coarse as a grazing photon's
                // vertical step, so the crossing fraction can round to 1 and leave no
                // remaining step: the photon would sit on the surface, count as in water and
                // exit a second time (a second transmission record, 1.5% of the photons at
                // 400 m with 0.05 ns bins). Place it just above the surface instead.
                ph.py = nextafterf(ys, 1.0e30f);
            }
        } else {
            // handle_seafloor
            float f = fminf(fmaxf((yf - ph.py) / svy, 0.f), 1.f);
            float xb = fmaf(f, svx, ph.px), yb = yf, zb = fmaf(f, svz, ph.pz);
            ph.sfi[0] = xb; ph.sfi[1] = yb; ph.sfi[2] = zb;
            if (PASS == ALB_FORWARD && out.hm_radius && ph.fwi[0] == ph.fwi[0]) {
                float ax = ph.fwi[0] - (float)sc.wc[0], az = ph.fwi[2] - (float)sc.wc[2];
                float bx = xb - (float)sc.fc[0], bz = zb - (float)sc.fc[2];
                int xi = (int)((sqrtf(ax * ax + az * az) / (float)sc.hm_wext) * sc.hm_bins);
                int yi = (int)((sqrtf(bx * bx + bz * bz) / (float)sc.hm_fext) * sc.hm_bins);
                if (xi >= 0 && xi < sc.hm_bins && yi >= 0 && yi < sc.hm_bins)
                    atomicAdd(out.hm_radius + xi * sc.hm_bins + yi, 1u);
            }
            emit_event_f<PASS>(out, ALB_BOTTOM_REFLECTION, kQueryBottom, ph, xb, yb, zb, ph.s, pid);
            // normalize(+y + isotropic unit vector): a cosine lobe about +y
            U4 b = src.block();
            float z = fmaf(-2.f, uf(b.x), 1.f);
            float r = sqrtf(fmaxf(0.f, 1.f - z * z));
            float sp, cp;
            __sincosf(6.283185307179586f * uf(b.y), &sp, &cp);
            float hx = r * cp, hy = 1.f + z, hz = r * sp;
            float hn = rsqrtf(fmaf(hx, hx, fmaf(hy, hy, hz * hz)));
            ph.dx = hx * hn; ph.dy = hy * hn; ph.dz = hz * hn;
            float rem = (1.f - f) * len;
            ph.px = fmaf(ph.dx, rem, xb); ph.py = fmaf(ph.dy, rem, yb); ph.pz = fmaf(ph.dz, rem, zb);
            const float a = water_alpha_f(sc, ph.py);
            if (sc.adjoint) {
                score_tau(sc, ph.sc, layer_of_f(sc, ph.py), a * len);
                ph.sc.l += sc.inv_albedo;
            }
            ph.tau = fmaf(a, len, ph.tau);
            ph.E *= sc.floor_albedo32;
        }
        ph.s += 1;
        ++events;
    }
}

template <int PASS>
ALB_DEVICE void emit_photon_fast(const SceneDev& sc, PhF& ph, PhiloxSrc& src) {
    const double* Rd = sc.rot_d;
    float R[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = (float)Rd[i];
    ph.px = ph.py = ph.pz = 0.f;
    ph.E = 1.f; ph.tau = 0.f; ph.taut = __int_as_float(0x7f800000); ph.s = 0;
    ph.sc = Score{0.f, 0.f, 0.f, 0.f};
    float qnan = __int_as_float(0x7fc00000);
    ph.fwi[0] = ph.fwi[1] = ph.fwi[2] = qnan;
    ph.sfi[0] = ph.sfi[1] = ph.sfi[2] = qnan;
    U4 b = src.block();
    if (PASS == ALB_FORWARD) {
        // once per photon: accurate logf / sincosf keep the beam footprint unquantised
        float th = (float)sc.rayleigh_sigma * sqrtf(-2.f * log1pf(-uf(b.x) * (float)sc.rayleigh_mass));
        float st, ct, sp, cp;
        sincosf(th, &st, &ct);
        sincospif(2.f * uf(b.y), &sp, &cp);
        float l0 = st * cp, l1 = st * sp, l2 = ct;
        ph.dx = l0 * R[0] + l1 * R[1] + l2 * R[2];
        ph.dy = l0 * R[3] + l1 * R[4] + l2 * R[5];
        ph.dz = l0 * R[6] + l1 * R[7] + l2 * R[8];
        float pulse = (float)sc.pulse_sigma32 * sqrtf(-2.f * logf(uf(b.z))) * cospif(2.f * uf(b.w));
        ph.t0 = pulse / (float)sc.eff_rate32;
    } else {
        float r = (float)sc.aperture * sqrtf(uf(b.x));
        float sa, ca;
        sincospif(2.f * uf(b.y), &sa, &ca);
        float d0 = r * ca, d1 = r * sa;
        float z = (float)sc.cos_fov + (1.f - (float)sc.cos_fov) * uf(b.z);
        float st = sqrtf(fmaxf(0.f, 1.f - z * z));
        float sp, cp;
        sincospif(2.f * uf(b.w), &sp, &cp);
        float l0 = st * cp, l1 = st * sp;
        // aperture point added to the direction, as the reference does
        ph.dx = (d0 * R[0] + d1 * R[1]) + (l0 * R[0] + l1 * R[1] + z * R[2]);
        ph.dy = (d0 * R[3] + d1 * R[4]) + (l0 * R[3] + l1 * R[4] + z * R[5]);
        ph.dz = (d0 * R[6] + d1 * R[7]) + (l0 * R[6] + l1 * R[7] + z * R[8]);
        ph.t0 = 0.f;
    }
}

}  // namespace alb
