/*
 * alb_oracle.c - CPU restatement of PyALBSim's photon-tracing / photon-mapping path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the parity checker of the GPU engine: only the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it. The product
 * path (pyalbsim_gb300) never calls it.
 *
 * Unlike the GPU tracer, which jumps from event to event, this oracle integrates every
 * photon step by step exactly as the reference's vectorised loop does for each photon:
 *   Simulation.simulate_batch            alb_sim/core/simulation.py:71-107
 *   simulate_photon_step/evaluate_state  alb_sim/core/simulation.py:220-322
 *   handle_water                         alb_sim/core/simulation.py:328-373
 *   handle_enter                         alb_sim/core/simulation.py:375-431
 *   handle_exit                          alb_sim/core/simulation.py:433-502
 *   handle_seafloor                      alb_sim/core/simulation.py:504-570
 *   emission                             alb_sim/physics/models/simulation.py:130-208
 *   scattering directions                alb_sim/physics/scatter/direction.py:7-51
 *   Rodrigues rotation                   alb_sim/math/rotation_matrix.py:39-102
 * and gathers with a brute-force exact k-NN (the reference uses scipy's KDTree, whose
 * answer is the same set) followed by the reference's weights in float64:
 *   sample_photons                       alb_sim/core/simulation.py:132-214
 *   GGX reflected energy                 alb_sim/physics/reflection/microfacet_brdf.py:18-147
 *   scatter bin energy                   alb_sim/physics/scatter/energy.py:8-52
 * Positions and directions are float64, energies and optical depths float32, matching the
 * dtypes the reference's arrays carry. Variates come either from a recorded replay
 * stream or from the same Philox4x32-10 streams and transforms the GPU uses.
 *
 * Pinned against the reference itself: tests/golden/make_golden.py runs the reference and
 * records its variates, photon maps, gather queries, waveforms, KDTree answers, 32-run
 * statistics and its own finite differences in albedo and roughness; the tests hold this
 * restatement to those fixtures record by record. The extensions the reference lacks
 * (path scores and the Jacobian, Henyey-Greenstein phase, fixed-radius gather, gated
 * windows, Gaussian surface slopes) are restated here from their definitions and pinned
 * by closed forms and differences instead.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/albgpu.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define NDIV ALB_PHASE_DIVISIONS
static const double TWO_PI = 6.283185307179586;
static const double PI = 3.141592653589793;
static const float EPS32 = 1.1920928955078125e-07f;

/* ------------------------------------------------------------------------------------ */
/* records                                                                              */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    int32_t channel; /* forward: record channel; backward: query kind 0 bottom 1 scatter 2 surface */
    int32_t photon;
    int64_t step;
    double pos[3];
    double dir[3];
    float energy;
    float time;
    float fwi[3];
    float sfi[3];
    float score[4]; /* adjoint path score d ln(p E)/d (a, b, g, albedo) of the prefix */
} OrRecord;

typedef struct {
    OrRecord* r;
    int64_t n, cap;
} OrBuf;

static void buf_push(OrBuf* b, const OrRecord* r) {
    if (b->n == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 1024;
        b->r = (OrRecord*)realloc(b->r, (size_t)b->cap * sizeof(OrRecord));
    }
    b->r[b->n++] = *r;
}

/* ------------------------------------------------------------------------------------ */
/* variates                                                                             */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    uint32_t x, y, z, w;
} U4;

static U4 philox(U4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        U4 n;
        n.x = (uint32_t)(p1 >> 32) ^ c.y ^ k0;
        n.y = (uint32_t)p1;
        n.z = (uint32_t)(p0 >> 32) ^ c.w ^ k1;
        n.w = (uint32_t)p0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

static double u01(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386963e-10; }

typedef struct {
    int replay;
    /* philox */
    uint32_t k0, k1, plo, phi, pass, ctr;
    /* replay */
    const double* v;
    const float* tau;
    int64_t pos, end;
    int* err;
} Src;

static U4 src_block(Src* s) {
    U4 c = {s->ctr, s->plo, s->phi, s->pass};
    s->ctr++;
    return philox(c, s->k0, s->k1);
}

static double src_next(Src* s) {
    if (s->pos < s->end) return s->v[s->pos++];
    *s->err = ALB_ERR_REPLAY;
    return 0.5;
}

static float src_next_tau(Src* s) {
    if (s->pos < s->end) return s->tau[s->pos++];
    *s->err = ALB_ERR_REPLAY;
    return 1.0f;
}

static float tau_of(double u) {
    float f = (float)u;
    return (float)(-log((double)f));
}

/* ------------------------------------------------------------------------------------ */
/* model helpers                                                                        */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    const AlbSceneParams* p;
    double eta, cos_fov, rs, rmass, ga2;
    float alb32;
    int64_t S;
} Model;

static int layer_of(const Model* m, double y) {
    double depth = -(y - m->p->surface_y);
    int i = 0;
    while (i < m->p->n_layers && !(m->p->layers[i].bottom_depth > depth)) ++i;
    return i < m->p->n_layers ? i : m->p->n_layers - 1;
}

static double norm3(double x, double y, double z) { return sqrt((x * x + y * y) + z * z); }

/* Depth-profiled layers (alb_sim/physics/models/water.py:85-101,190-245,306-308;
 * utils/parameter_profile.py:46-99): local depth below the layer top (float32 offset),
 * LinearParameter in float32 at t = float32(z / h), ExponentialParameter in float64, the
 * attenuation by numpy.interp on the float32-depth LUT at float32(z). */
static double profile_value(int kind, double p0, double p1, double z, double h) {
    if (kind == 1) {
        float t = (float)(z / h);
        float d = (float)(p1 - p0);
        float prod = t * d;
        return (double)((float)p0 + prod);
    }
    if (kind == 2) {
        double l0 = log(p0), l1 = log(p1);
        return exp(l0 + (z / h) * (l1 - l0));
    }
    return p0;
}

static double local_depth(const Model* m, int L, double y) {
    return -(y - m->p->surface_y) - m->p->layers[L].top32;
}

static double lut_alpha(const AlbLayer* L, double z) {
    const float* xp = L->lut_z;
    const double* fp = L->lut_alpha;
    int n = L->lut_n;
    double x = (double)(float)z;
    if (!(x >= (double)xp[0])) return fp[0];
    if (x >= (double)xp[n - 1]) return fp[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if ((double)xp[mid] <= x) lo = mid;
        else hi = mid;
    }
    if (x == (double)xp[lo]) return fp[lo];
    double slope = (fp[lo + 1] - fp[lo]) / ((double)xp[lo + 1] - (double)xp[lo]);
    double prod = slope * (x - (double)xp[lo]);
    return prod + fp[lo];
}

/* speed of a water step starting at height y */
static double water_speed(const Model* m, double y) {
    int L = layer_of(m, y);
    const AlbLayer* A = &m->p->layers[L];
    if (!A->profiled) return A->speed;
    double n = profile_value(A->n_kind, A->n_start, A->n_end, local_depth(m, L, y), A->height);
    if (A->n_kind == 1) {
        float q = 299800000.0f / (float)n;
        return (double)q;
    }
    return (double)(float)(299800000.0 / n);
}

static float water_alpha(const Model* m, double y) {
    int L = layer_of(m, y);
    const AlbLayer* A = &m->p->layers[L];
    if (!A->profiled) return A->alpha;
    return (float)lut_alpha(A, local_depth(m, L, y));
}

static float water_ssa(const Model* m, double y) {
    int L = layer_of(m, y);
    const AlbLayer* A = &m->p->layers[L];
    if (!A->profiled) return A->ssa;
    double z = local_depth(m, L, y);
    double al = lut_alpha(A, z);
    double a = profile_value(A->a_kind, A->a_start, A->a_end, z, A->height);
    return (float)((al - a) / al);
}

static double schlick(double f0, double c) { return f0 + (1.0 - f0) * pow(1.0 - c, 5.0); }

/* numpy.interp(u, cdf, theta) */
/* numpy.interp(u, cdf, theta); *interval gets the table interval of the result: 0 below
 * cdf[0], i + 1 for cdf[i] <= u < cdf[i + 1] (the index of dlog_sample_g, the score of an
 * angle drawn from the tabulated CDF) */
static double interp(const AlbLayer* L, double u, int* interval) {
    const double* xp = L->phase_cdf;
    const double* fp = L->phase_theta;
    *interval = 0;
    if (u < xp[0]) return fp[0];
    *interval = NDIV - 1;
    if (u >= xp[NDIV - 1]) return fp[NDIV - 1];
    int lo = 0, hi = NDIV - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (xp[mid] <= u) lo = mid; else hi = mid;
    }
    *interval = lo + 1;
    if (u == xp[lo]) return fp[lo];
    double slope = (fp[lo + 1] - fp[lo]) / (xp[lo + 1] - xp[lo]);
    return slope * (u - xp[lo]) + fp[lo];
}

/* rotation_from_z_batch for one vector (float32 matrix), applied to l */
static void rot_apply(const double d[3], const double l[3], double out[3]) {
    double n = norm3(d[0], d[1], d[2]);
    double v[3] = {d[0] / n, d[1] / n, d[2] / n};
    double c = v[2];
    if (fabs(c - 1.0) <= 1e-08 + 1e-05 * fabs(1.0)) {
        out[0] = l[0]; out[1] = l[1]; out[2] = l[2];
        return;
    }
    if (fabs(c - -1.0) <= 1e-08 + 1e-05 * fabs(-1.0)) {
        out[0] = l[0]; out[1] = -l[1]; out[2] = -l[2];
        return;
    }
    double vx = -v[1], vy = v[0];
    double s2 = vx * vx + vy * vy;
    double K[3][3] = {{0.0, -0.0, vy}, {0.0, 0.0, -vx}, {-vy, vx, 0.0}};
    double R[3][3];
    double f = (1.0 - c) / s2;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double kk = 0.0;
            for (int t = 0; t < 3; ++t) kk += K[i][t] * K[t][j];
            double e = ((i == j ? 1.0 : 0.0) + K[i][j]) + kk * f;
            R[i][j] = (double)(float)e;
        }
    for (int i = 0; i < 3; ++i) out[i] = (R[i][0] * l[0] + R[i][1] * l[1]) + R[i][2] * l[2];
}

/* ------------------------------------------------------------------------------------ */
/* one photon, step by step                                                             */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    double p[3], d[3];
    float E, tau, taut, t0;
    float fwi[3], sfi[3];
    double sc[4]; /* adjoint path score (extension) */
} Ph;

/* Adjoint scores (extension, no counterpart in the reference). The scatter process is
 * Poisson in the optical depth tau: each increment dtau in layer L multiplies the path
 * density by e^(-dtau), each scatter by alpha_L, so d ln p / d theta gains
 * -dtau d ln(alpha_L)/d theta per increment and +d ln(alpha_L)/d theta per scatter; the
 * energy gains d ln(ssa_L)/d theta per scatter and 1/albedo per seafloor reflection; an
 * HG layer's direction sampling adds d ln p_HG(mu)/dg. */
static void score_tau(const AlbSceneParams* P, Ph* ph, int L, double dtau) {
    for (int i = 0; i < 3; ++i) ph->sc[i] -= dtau * P->layers[L].dlog_alpha[i];
}
static double hg_dlogp(double g, double mu) {
    return -2.0 * g / (1.0 - g * g) - 3.0 * (g - mu) / (1.0 + g * g - 2.0 * g * mu);
}

static void emit(const Model* m, int pass, Src* s, Ph* ph) {
    const float* Rf = m->p->laser_rot;
    double R[9];
    for (int i = 0; i < 9; ++i) R[i] = (double)Rf[i];
    ph->p[0] = ph->p[1] = ph->p[2] = 0.0;
    ph->E = 1.0f;
    ph->tau = 0.0f;
    ph->taut = INFINITY;
    for (int i = 0; i < 4; ++i) ph->sc[i] = 0.0;
    ph->fwi[0] = ph->fwi[1] = ph->fwi[2] = NAN;
    ph->sfi[0] = ph->sfi[1] = ph->sfi[2] = NAN;
    if (pass == ALB_FORWARD) {
        double th, phi, pulse;
        if (s->replay) {
            th = src_next(s);
            phi = src_next(s);
            pulse = src_next(s);
        } else {
            U4 b = src_block(s);
            th = m->rs * sqrt(-2.0 * log(1.0 - u01(b.x) * m->rmass));
            phi = TWO_PI * u01(b.y);
            pulse = m->p->pulse_sigma * (sqrt(-2.0 * log(u01(b.z))) * cos(TWO_PI * u01(b.w)));
        }
        double st = sin(th), ct = cos(th);
        double l[3] = {st * cos(phi), st * sin(phi), ct};
        for (int i = 0; i < 3; ++i)
            ph->d[i] = (double)(float)((l[0] * R[3 * i] + l[1] * R[3 * i + 1]) + l[2] * R[3 * i + 2]);
        ph->t0 = (float)pulse / (float)m->p->effective_rate;
    } else {
        double x1, x2, z, phc;
        if (s->replay) {
            x1 = src_next(s);
            x2 = src_next(s);
            z = src_next(s);
            phc = src_next(s);
        } else {
            U4 b = src_block(s);
            x1 = u01(b.x);
            x2 = u01(b.y);
            z = m->cos_fov + (1.0 - m->cos_fov) * u01(b.z);
            phc = TWO_PI * u01(b.w);
        }
        double r = m->p->aperture_radius * sqrt(x1);
        double a = TWO_PI * x2;
        double dl[3] = {r * cos(a), r * sin(a), 0.0};
        double st = sqrt(1.0 - z * z);
        double l[3] = {st * cos(phc), st * sin(phc), z};
        for (int i = 0; i < 3; ++i) {
            double disk = (dl[0] * R[3 * i] + dl[1] * R[3 * i + 1]) + dl[2] * R[3 * i + 2];
            float cone = (float)((l[0] * R[3 * i] + l[1] * R[3 * i + 1]) + l[2] * R[3 * i + 2]);
            ph->d[i] = disk + (double)cone;
        }
        ph->t0 = 0.0f;
    }
}

static void record(OrBuf* out, int channel, int photon, int64_t step, const double pos[3], const Ph* ph) {
    OrRecord r;
    r.channel = channel;
    r.photon = photon;
    r.step = step;
    for (int i = 0; i < 3; ++i) {
        r.pos[i] = pos[i];
        r.dir[i] = ph->d[i];
        r.fwi[i] = ph->fwi[i];
        r.sfi[i] = ph->sfi[i];
    }
    r.energy = ph->E;
    r.time = ph->t0 + (float)step;
    for (int i = 0; i < 4; ++i) r.score[i] = (float)ph->sc[i];
    buf_push(out, &r);
}

/* Extension (the reference's surface is flat): Gaussian surface slopes. Facet normal
 * normalize(-gx, 1, -gz), gx, gz ~ N(0, sigma^2) from one Box-Muller block; a facet facing
 * away from the photon, or one sending it to the wrong side, falls back to the flat surface. */
static void draw_facet(const AlbSceneParams* P, Src* s, double mf[3]) {
    U4 b = src_block(s);
    double r0 = sqrt(-2.0 * log(u01(b.x))), a0 = TWO_PI * u01(b.y);
    double gx = r0 * cos(a0) * P->slope_sigma, gz = r0 * sin(a0) * P->slope_sigma;
    double nn = norm3(gx, 1.0, gz);
    mf[0] = -gx / nn;
    mf[1] = 1.0 / nn;
    mf[2] = -gz / nn;
}

static void trace_one(const Model* m, int pass, Src* s, Ph* ph, int photon, OrBuf* out, unsigned* hm_radius) {
    const AlbSceneParams* P = m->p;
    const double ys = P->surface_y, yf = P->floor_y, dt = P->dt;
    for (int64_t step = 0; step < m->S; ++step) {
        double v = (ph->p[1] > ys) ? P->speed_air : water_speed(m, ph->p[1]);
        double nx[3];
        for (int i = 0; i < 3; ++i) nx[i] = ph->p[i] + (ph->d[i] * v) * dt;
        double y = ph->p[1], yn = nx[1];
        int st = 0; /* 0 air, 1 enter, 2 water, 3 floor, 4 exit */
        if (y > ys && yn <= ys) st = 1;
        if (y <= ys && yn > yf) st = 2;
        if (y > yf && yn <= yf) st = 3;
        if (y <= ys && yn > ys) st = 4;
        if (st == 0) {
            for (int i = 0; i < 3; ++i) ph->p[i] = nx[i];
            continue;
        }
        double sv[3] = {nx[0] - ph->p[0], nx[1] - ph->p[1], nx[2] - ph->p[2]};
        double len = norm3(sv[0], sv[1], sv[2]);
        if (st == 2) {
            float a = water_alpha(m, ph->p[1]);
            score_tau(P, ph, layer_of(m, ph->p[1]), (double)a * len);
            ph->tau = (float)((double)ph->tau + (double)a * len);
            int scatter = ph->tau >= ph->taut;
            for (int i = 0; i < 3; ++i) ph->p[i] = nx[i];
            if (scatter) {
                int L = layer_of(m, ph->p[1]);
                for (int i = 0; i < 3; ++i) ph->sc[i] += P->layers[L].dlog_alpha[i];
                record(out, pass == ALB_FORWARD ? ALB_SCATTER : 1, photon, step, ph->p, ph);
                double uth, phi;
                float nt;
                if (s->replay) {
                    uth = src_next(s);
                    phi = src_next(s);
                    nt = src_next_tau(s);
                } else {
                    U4 b = src_block(s);
                    uth = u01(b.x);
                    phi = TWO_PI * u01(b.y);
                    nt = tau_of(u01(b.z));
                }
                int interval;
                double th = interp(&P->layers[L], uth, &interval);
                double lv[3] = {sin(th) * cos(phi), sin(th) * sin(phi), cos(th)};
                double nd[3];
                rot_apply(ph->d, lv, nd);
                for (int i = 0; i < 3; ++i) ph->d[i] = nd[i];
                for (int i = 0; i < 3; ++i) ph->sc[i] += P->layers[L].dlog_ssa[i];
                if (P->layers[L].hg_g != 0.0)
                    ph->sc[2] += P->layers[L].dlog_sample_g ? P->layers[L].dlog_sample_g[interval]
                                                            : hg_dlogp(P->layers[L].hg_g, cos(th));
                ph->E = ph->E * water_ssa(m, ph->p[1]);
                ph->tau = ph->tau - ph->taut;
                ph->taut = nt;
            }
            continue;
        }
        double plane = (st == 3) ? yf : ys;
        double f = (plane - ph->p[1]) / sv[1];
        f = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
        double xs[3];
        for (int i = 0; i < 3; ++i) xs[i] = ph->p[i] + f * sv[i];
        double rem = (1.0 - f) * len;
        if (st == 1) {
            for (int i = 0; i < 3; ++i) ph->fwi[i] = (float)xs[i];
            double F = schlick(P->f0, -ph->d[1]);
            record(out, pass == ALB_FORWARD ? ALB_SURFACE_REFLECTION : 2, photon, step, xs, ph);
            int flat = 1;
            if (P->slope_sigma > 0.0) {
                double mf[3];
                draw_facet(P, s, mf);
                double cf = -(ph->d[0] * mf[0] + ph->d[1] * mf[1] + ph->d[2] * mf[2]);
                if (cf > 0.0) {
                    cf = cf > 1.0 ? 1.0 : cf;
                    double ctf = sqrt(fmax(0.0, 1.0 - (m->eta * m->eta) * (1.0 - cf * cf)));
                    double k = m->eta * cf - ctf;
                    double t[3];
                    for (int i = 0; i < 3; ++i) t[i] = m->eta * ph->d[i] + k * mf[i];
                    if (t[1] < 0.0) {
                        double tn = norm3(t[0], t[1], t[2]);
                        for (int i = 0; i < 3; ++i) ph->d[i] = t[i] / tn;
                        F = schlick(P->f0, cf);
                        flat = 0;
                    }
                }
            }
            if (flat) {
                double ci = -ph->d[1];
                ci = ci < -1.0 ? -1.0 : (ci > 1.0 ? 1.0 : ci);
                double sin2 = (m->eta * m->eta) * (1.0 - ci * ci);
                double ct = sqrt(fmax(0.0, 1.0 - sin2));
                double t[3] = {m->eta * ph->d[0], m->eta * ph->d[1] + (m->eta * ci - ct), m->eta * ph->d[2]};
                double tn = norm3(t[0], t[1], t[2]);
                for (int i = 0; i < 3; ++i) ph->d[i] = t[i] / tn;
            }
            ph->E = (float)((double)ph->E * (1.0 - F));
            for (int i = 0; i < 3; ++i) ph->p[i] = xs[i] + ph->d[i] * rem;
            ph->taut = s->replay ? src_next_tau(s) : tau_of(u01(src_block(s).x));
        } else if (st == 4) {
            double mf[3] = {0.0, 1.0, 0.0}, cf = ph->d[1];
            int tilted = 0;
            if (P->slope_sigma > 0.0) {
                draw_facet(P, s, mf);
                cf = ph->d[0] * mf[0] + ph->d[1] * mf[1] + ph->d[2] * mf[2];
                tilted = cf > 0.0;
                if (!tilted) {
                    mf[0] = 0.0; mf[1] = 1.0; mf[2] = 0.0;
                    cf = ph->d[1];
                }
            }
            double F = schlick(P->f0, tilted ? (cf > 1.0 ? 1.0 : cf) : ph->d[1]);
            double U = s->replay ? src_next(s) : u01(src_block(s).x);
            int reflect = U < F;
            if (pass == ALB_FORWARD && !reflect) record(out, ALB_SURFACE_TRANSMISSION_UP, photon, step, xs, ph);
            double ci = tilted ? cf : ph->d[1];
            ci = ci < -1.0 ? -1.0 : (ci > 1.0 ? 1.0 : ci);
            double sin2 = (m->eta * m->eta) * (1.0 - ci * ci);
            double ct = sqrt(fmax(0.0, 1.0 - sin2));
            if (sin2 > 1.0) reflect = 1;
            int done = 0;
            if (tilted) {
                if (reflect) {
                    double r[3];
                    for (int i = 0; i < 3; ++i) r[i] = ph->d[i] - 2.0 * cf * mf[i];
                    if (r[1] < 0.0) {
                        for (int i = 0; i < 3; ++i) ph->d[i] = r[i];
                        done = 1;
                    }
                } else {
                    double k = m->eta * ci - ct, t[3];
                    for (int i = 0; i < 3; ++i) t[i] = m->eta * ph->d[i] - k * mf[i];
                    if (t[1] > 0.0) {
                        double tn = norm3(t[0], t[1], t[2]);
                        for (int i = 0; i < 3; ++i) ph->d[i] = t[i] / tn;
                        done = 1;
                    }
                }
            }
            if (!done) {
                if (reflect) {
                    ph->d[1] = -ph->d[1];
                } else {
                    double c0 = ph->d[1];
                    c0 = c0 < -1.0 ? -1.0 : (c0 > 1.0 ? 1.0 : c0);
                    double ct0 = sqrt(fmax(0.0, 1.0 - (m->eta * m->eta) * (1.0 - c0 * c0)));
                    double t[3] = {m->eta * ph->d[0], m->eta * ph->d[1] - (m->eta * c0 - ct0), m->eta * ph->d[2]};
                    double tn = norm3(t[0], t[1], t[2]);
                    for (int i = 0; i < 3; ++i) ph->d[i] = t[i] / tn;
                }
            }
            for (int i = 0; i < 3; ++i) ph->p[i] = xs[i] + ph->d[i] * rem;
            if (reflect) {
                float a = water_alpha(m, ph->p[1]);
                score_tau(P, ph, layer_of(m, ph->p[1]), (double)a * len);
                ph->tau = (float)((double)ph->tau + (double)a * len);
            }
        } else { /* seafloor */
            for (int i = 0; i < 3; ++i) ph->sfi[i] = (float)xs[i];
            if (pass == ALB_FORWARD && hm_radius && !isnan(ph->fwi[0])) {
                double ax = (double)ph->fwi[0] - P->water_center[0], az = (double)ph->fwi[2] - P->water_center[2];
                double bx = xs[0] - P->floor_center[0], bz = xs[2] - P->floor_center[2];
                double rs = sqrt(ax * ax + az * az), rf = sqrt(bx * bx + bz * bz);
                long long xi = (long long)((rs / P->heatmap_water_extent) * P->heatmap_bins);
                long long yi = (long long)((rf / P->heatmap_floor_extent) * P->heatmap_bins);
                if (xi >= 0 && xi < P->heatmap_bins && yi >= 0 && yi < P->heatmap_bins) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                    hm_radius[xi * P->heatmap_bins + yi] += 1u;
                }
            }
            record(out, pass == ALB_FORWARD ? ALB_BOTTOM_REFLECTION : 0, photon, step, xs, ph);
            double n0, n1, n2;
            if (s->replay) {
                n0 = src_next(s);
                n1 = src_next(s);
                n2 = src_next(s);
            } else {
                U4 b = src_block(s);
                double r0 = sqrt(-2.0 * log(u01(b.x))), a0 = TWO_PI * u01(b.y);
                double r1 = sqrt(-2.0 * log(u01(b.z))), a1 = TWO_PI * u01(b.w);
                n0 = r0 * cos(a0);
                n1 = r0 * sin(a0);
                n2 = r1 * cos(a1);
            }
            float g0 = (float)n0, g1 = (float)n1, g2 = (float)n2;
            volatile float gq = (g0 * g0 + g1 * g1) + g2 * g2;
            float gn = sqrtf(gq);
            g0 = g0 / gn; g1 = g1 / gn; g2 = g2 / gn;
            double h[3] = {(double)g0, 1.0 + (double)g1, (double)g2};
            double hn = norm3(h[0], h[1], h[2]);
            for (int i = 0; i < 3; ++i) ph->d[i] = h[i] / hn;
            for (int i = 0; i < 3; ++i) ph->p[i] = xs[i] + ph->d[i] * rem;
            float a = water_alpha(m, ph->p[1]);
            score_tau(P, ph, layer_of(m, ph->p[1]), (double)a * len);
            if (P->seafloor_albedo > 0.0) ph->sc[3] += 1.0 / P->seafloor_albedo;
            ph->tau = (float)((double)ph->tau + (double)a * len);
            ph->E = ph->E * m->alb32;
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* exported: tracing                                                                    */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    OrRecord* records; /* owned; free with oracle_free */
    int64_t n_records;
    double* exit_pd;   /* n * 6: pos, dir */
    float* exit_f;     /* n * 10: energy, tau, tau_target, time, fwi[3], sfi[3] */
    unsigned* hm_radius;
} OracleTrace;

static void init_model(Model* m, const AlbSceneParams* p) {
    m->p = p;
    m->eta = 1.0 / p->n_water;
    m->cos_fov = cos(p->fov);
    m->rs = p->divergence / 3.0;
    m->rmass = -expm1(-(p->divergence * p->divergence) / (2.0 * m->rs * m->rs));
    m->alb32 = (float)p->seafloor_albedo;
    m->S = p->steps * (int64_t)p->sample_multiplier;
}

int oracle_record_size(void) { return (int)sizeof(OrRecord); }

/* Trace n photons of one pass. Records (forward) / queries (backward) are returned in
 * (photon, step) order. hm_radius (nullable) accumulates the scatter-radius heatmap. */
int oracle_trace(const AlbSceneParams* p, int pass, uint64_t n, uint64_t seed, uint64_t first,
                 const int64_t* offsets, const double* values, const float* tau, OracleTrace* out, int threads) {
    Model m;
    init_model(&m, p);
    int err = 0;
    OrBuf* bufs = (OrBuf*)calloc((size_t)n ? n : 1, sizeof(OrBuf));
    out->exit_pd = (double*)malloc((size_t)(n ? n : 1) * 6 * sizeof(double));
    out->exit_f = (float*)malloc((size_t)(n ? n : 1) * 10 * sizeof(float));
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        Src s;
        memset(&s, 0, sizeof s);
        int perr = 0;
        s.err = &perr;
        uint64_t gid = first + (uint64_t)i;
        if (offsets) {
            s.replay = 1;
            s.v = values;
            s.tau = tau;
            s.pos = offsets[i];
            s.end = offsets[i + 1];
        } else {
            s.k0 = (uint32_t)seed;
            s.k1 = (uint32_t)(seed >> 32);
            s.plo = (uint32_t)gid;
            s.phi = (uint32_t)(gid >> 32);
            s.pass = (uint32_t)pass;
        }
        Ph ph;
        emit(&m, pass, &s, &ph);
        trace_one(&m, pass, &s, &ph, (int)gid, &bufs[i], out->hm_radius);
        double* pd = out->exit_pd + 6 * i;
        for (int k = 0; k < 3; ++k) {
            pd[k] = ph.p[k];
            pd[3 + k] = ph.d[k];
        }
        float* f = out->exit_f + 10 * i;
        f[0] = ph.E; f[1] = ph.tau; f[2] = ph.taut; f[3] = ph.t0;
        for (int k = 0; k < 3; ++k) {
            f[4 + k] = ph.fwi[k];
            f[7 + k] = ph.sfi[k];
        }
        if (perr) err = perr;
    }
    int64_t total = 0;
    for (uint64_t i = 0; i < n; ++i) total += bufs[i].n;
    out->records = (OrRecord*)malloc((size_t)(total ? total : 1) * sizeof(OrRecord));
    int64_t at = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (bufs[i].n) memcpy(out->records + at, bufs[i].r, (size_t)bufs[i].n * sizeof(OrRecord));
        at += bufs[i].n;
        free(bufs[i].r);
    }
    free(bufs);
    out->n_records = total;
    return err;
}

void oracle_free(OracleTrace* t) {
    free(t->records);
    free(t->exit_pd);
    free(t->exit_f);
    t->records = NULL;
    t->exit_pd = NULL;
    t->exit_f = NULL;
}

/* ------------------------------------------------------------------------------------ */
/* exported: gather                                                                     */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    double d2;
    int32_t i;
} Cand;

static void heap_down(Cand* h, int n, int i) {
    for (;;) {
        int l = 2 * i + 1, r = l + 1, b = i;
        if (l < n && (h[l].d2 > h[b].d2 || (h[l].d2 == h[b].d2 && h[l].i > h[b].i))) b = l;
        if (r < n && (h[r].d2 > h[b].d2 || (h[r].d2 == h[b].d2 && h[r].i > h[b].i))) b = r;
        if (b == i) return;
        Cand t = h[i];
        h[i] = h[b];
        h[b] = t;
        i = b;
    }
}

static int cand_cmp(const void* a, const void* b) {
    const Cand* x = (const Cand*)a;
    const Cand* y = (const Cand*)b;
    if (x->d2 < y->d2) return -1;
    if (x->d2 > y->d2) return 1;
    return (x->i > y->i) - (x->i < y->i);
}

/* Exact k nearest (float64 distances of float32 points), sorted ascending. */
static void knn_brute(const float* pts, int64_t m, const double q[3], int k, Cand* out) {
    int n = 0;
    for (int64_t j = 0; j < m; ++j) {
        double dx = (double)pts[3 * j] - q[0], dy = (double)pts[3 * j + 1] - q[1], dz = (double)pts[3 * j + 2] - q[2];
        double d2 = (dx * dx + dy * dy) + dz * dz;
        if (n < k) {
            out[n].d2 = d2;
            out[n].i = (int32_t)j;
            ++n;
            if (n == k)
                for (int t = k / 2 - 1; t >= 0; --t) heap_down(out, k, t);
        } else if (d2 < out[0].d2) {
            out[0].d2 = d2;
            out[0].i = (int32_t)j;
            heap_down(out, k, 0);
        }
    }
    qsort(out, (size_t)k, sizeof(Cand), cand_cmp);
}

/* k-d tree over the float32 points of a map, for the exact k-NN the reference takes from
 * scipy's KDTree (photon_mapping/photon_map_index.py:17, core/simulation.py:139-142). It
 * returns what knn_brute returns: the k smallest (float64 squared distance, index) pairs,
 * sorted. A point replaces the current k-th when its pair is smaller, and a subtree is
 * skipped only when the float64 lower bound of its box is strictly above the k-th distance
 * (the bound is formed with the same operations as a point's distance, so rounding keeps it
 * at or below the distance of every point inside). Ties at the k-th distance therefore go
 * to the smaller index, whatever order the tree visits the points in. */
#define KD_LEAF 16
typedef struct {
    int32_t* perm;
    int64_t nnodes, cap;
    float* box;       /* 6 per node: lo xyz, hi xyz */
    int64_t* range;   /* 2 per node: begin, end in perm */
    int64_t* child;   /* 2 per node: left, right (-1: leaf) */
} KdTree;

static double coord(const float* pts, int32_t i, int a) { return (double)pts[3 * (int64_t)i + a]; }

static void kd_select(const float* pts, int32_t* v, int64_t lo, int64_t hi, int64_t nth, int a) {
    /* quickselect: v[nth] in sorted position by (coordinate a, index) */
    while (hi - lo > 1) {
        int32_t pv = v[lo + (hi - lo) / 2];
        double pc = coord(pts, pv, a);
        int64_t i = lo, j = hi - 1;
        while (i <= j) {
            while (coord(pts, v[i], a) < pc || (coord(pts, v[i], a) == pc && v[i] < pv)) ++i;
            while (coord(pts, v[j], a) > pc || (coord(pts, v[j], a) == pc && v[j] > pv)) --j;
            if (i <= j) {
                int32_t t = v[i];
                v[i] = v[j];
                v[j] = t;
                ++i;
                --j;
            }
        }
        if (nth <= j) hi = j + 1;
        else if (nth >= i) lo = i;
        else return;
    }
}

static int64_t kd_build_node(KdTree* t, const float* pts, int64_t b, int64_t e) {
    if (t->nnodes == t->cap) {
        t->cap *= 2;
        t->box = (float*)realloc(t->box, (size_t)t->cap * 6 * sizeof(float));
        t->range = (int64_t*)realloc(t->range, (size_t)t->cap * 2 * sizeof(int64_t));
        t->child = (int64_t*)realloc(t->child, (size_t)t->cap * 2 * sizeof(int64_t));
    }
    int64_t id = t->nnodes++;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = b; i < e; ++i)
        for (int a = 0; a < 3; ++a) {
            float v = pts[3 * (int64_t)t->perm[i] + a];
            if (v < lo[a]) lo[a] = v;
            if (v > hi[a]) hi[a] = v;
        }
    for (int a = 0; a < 3; ++a) {
        t->box[6 * id + a] = lo[a];
        t->box[6 * id + 3 + a] = hi[a];
    }
    t->range[2 * id] = b;
    t->range[2 * id + 1] = e;
    t->child[2 * id] = t->child[2 * id + 1] = -1;
    if (e - b > KD_LEAF) {
        int ax = 0;
        for (int a = 1; a < 3; ++a)
            if (hi[a] - lo[a] > hi[ax] - lo[ax]) ax = a;
        int64_t mid = b + (e - b) / 2;
        kd_select(pts, t->perm, b, e, mid, ax);
        int64_t l = kd_build_node(t, pts, b, mid);
        int64_t r = kd_build_node(t, pts, mid, e);
        t->child[2 * id] = l;
        t->child[2 * id + 1] = r;
    }
    return id;
}

static KdTree* kd_build(const float* pts, int64_t m) {
    KdTree* t = (KdTree*)calloc(1, sizeof(KdTree));
    t->perm = (int32_t*)malloc((size_t)(m > 0 ? m : 1) * sizeof(int32_t));
    for (int64_t i = 0; i < m; ++i) t->perm[i] = (int32_t)i;
    t->cap = 64;
    t->box = (float*)malloc((size_t)t->cap * 6 * sizeof(float));
    t->range = (int64_t*)malloc((size_t)t->cap * 2 * sizeof(int64_t));
    t->child = (int64_t*)malloc((size_t)t->cap * 2 * sizeof(int64_t));
    if (m > 0) kd_build_node(t, pts, 0, m);
    return t;
}

static void kd_free(KdTree* t) {
    if (!t) return;
    free(t->perm);
    free(t->box);
    free(t->range);
    free(t->child);
    free(t);
}

static double kd_box_d2(const KdTree* t, int64_t node, const double q[3]) {
    double g[3];
    for (int a = 0; a < 3; ++a) {
        double lo = (double)t->box[6 * node + a] - q[a], hi = q[a] - (double)t->box[6 * node + 3 + a];
        g[a] = lo > 0.0 ? lo : (hi > 0.0 ? hi : 0.0);
    }
    return (g[0] * g[0] + g[1] * g[1]) + g[2] * g[2];
}

static void kd_knn_node(const KdTree* t, const float* pts, int64_t node, const double q[3], int k, Cand* h, int* n) {
    if (t->child[2 * node] < 0) {
        for (int64_t i = t->range[2 * node]; i < t->range[2 * node + 1]; ++i) {
            const int32_t j = t->perm[i];
            double dx = (double)pts[3 * (int64_t)j] - q[0], dy = (double)pts[3 * (int64_t)j + 1] - q[1],
                   dz = (double)pts[3 * (int64_t)j + 2] - q[2];
            double d2 = (dx * dx + dy * dy) + dz * dz;
            if (*n < k) {
                h[*n].d2 = d2;
                h[*n].i = j;
                ++*n;
                if (*n == k)
                    for (int s = k / 2 - 1; s >= 0; --s) heap_down(h, k, s);
            } else if (d2 < h[0].d2 || (d2 == h[0].d2 && j < h[0].i)) {
                h[0].d2 = d2;
                h[0].i = j;
                heap_down(h, k, 0);
            }
        }
        return;
    }
    int64_t c0 = t->child[2 * node], c1 = t->child[2 * node + 1];
    double b0 = kd_box_d2(t, c0, q), b1 = kd_box_d2(t, c1, q);
    if (b1 < b0) {
        int64_t tc = c0;
        c0 = c1;
        c1 = tc;
        double tb = b0;
        b0 = b1;
        b1 = tb;
    }
    if (*n < k || b0 <= h[0].d2) kd_knn_node(t, pts, c0, q, k, h, n);
    if (*n < k || b1 <= h[0].d2) kd_knn_node(t, pts, c1, q, k, h, n);
}

/* Exact k nearest through the tree, sorted ascending (the same array knn_brute gives). */
static void knn_tree(const KdTree* t, const float* pts, const double q[3], int k, Cand* out) {
    int n = 0;
    kd_knn_node(t, pts, 0, q, k, out, &n);
    qsort(out, (size_t)k, sizeof(Cand), cand_cmp);
}

/* Every point with float64 squared distance <= R2, in ascending index order (the order the
 * brute-force scan produces, so float64 sums over them are unchanged). */
static int cand_idx_cmp(const void* a, const void* b) {
    const Cand* x = (const Cand*)a;
    const Cand* y = (const Cand*)b;
    return (x->i > y->i) - (x->i < y->i);
}
static void kd_range_node(const KdTree* t, const float* pts, int64_t node, const double q[3], double R2, Cand** c,
                          int64_t* cnt, int64_t* cap) {
    if (kd_box_d2(t, node, q) > R2) return;
    if (t->child[2 * node] < 0) {
        for (int64_t i = t->range[2 * node]; i < t->range[2 * node + 1]; ++i) {
            const int32_t j = t->perm[i];
            double dx = (double)pts[3 * (int64_t)j] - q[0], dy = (double)pts[3 * (int64_t)j + 1] - q[1],
                   dz = (double)pts[3 * (int64_t)j + 2] - q[2];
            if ((dx * dx + dy * dy) + dz * dz <= R2) {
                if (*cnt == *cap) {
                    *cap *= 2;
                    *c = (Cand*)realloc(*c, (size_t)*cap * sizeof(Cand));
                }
                (*c)[*cnt].i = j;
                (*c)[*cnt].d2 = 0.0;
                ++*cnt;
            }
        }
        return;
    }
    kd_range_node(t, pts, t->child[2 * node], q, R2, c, cnt, cap);
    kd_range_node(t, pts, t->child[2 * node + 1], q, R2, c, cnt, cap);
}

/* 1: every k-NN and radius query scans all points (the checker); 0: the k-d tree. */
static int g_knn_brute = 0;
void oracle_set_knn_brute(int on) { g_knn_brute = on; }

int oracle_knn(const float* pts, int64_t m, const double* qs, int64_t nq, int k, int32_t* idx, double* dist,
               int threads) {
    if (m < k) return ALB_ERR_TOO_FEW;
    KdTree* tree = g_knn_brute ? NULL : kd_build(pts, m);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 8)
#endif
    for (int64_t i = 0; i < nq; ++i) {
        Cand* c = (Cand*)malloc((size_t)k * sizeof(Cand));
        if (tree) knn_tree(tree, pts, qs + 3 * i, k, c);
        else knn_brute(pts, m, qs + 3 * i, k, c);
        for (int j = 0; j < k; ++j) {
            idx[i * k + j] = c[j].i;
            dist[i * k + j] = sqrt(c[j].d2);
        }
        free(c);
    }
    kd_free(tree);
    return 0;
}

/* GGX reflected energy with wi (per neighbour) and wo, normal +y, in float64 */
static double ggx(double rough, double f0, const double wi_in[3], const double wo_in[3]) {
    double wn = norm3(wi_in[0], wi_in[1], wi_in[2]);
    double wi[3] = {wi_in[0] / wn, wi_in[1] / wn, wi_in[2] / wn};
    double on = norm3(wo_in[0], wo_in[1], wo_in[2]);
    double wo[3] = {wo_in[0] / on, wo_in[1] / on, wo_in[2] / on};
    double h[3] = {wi[0] + wo[0], wi[1] + wo[1], wi[2] + wo[2]};
    double hn = norm3(h[0], h[1], h[2]);
    if (hn == 0.0) hn = 1.0;
    for (int i = 0; i < 3; ++i) h[i] /= hn;
    double a = rough * rough;
    double n_wi = wi[1] < 0 ? 0 : (wi[1] > 1 ? 1 : wi[1]);
    double n_wo = wo[1] < 0 ? 0 : (wo[1] > 1 ? 1 : wo[1]);
    double wih = (wi[0] * h[0] + wi[1] * h[1]) + wi[2] * h[2];
    wih = wih < 0 ? 0 : (wih > 1 ? 1 : wih);
    double nh = h[1] < 0 ? 0 : (h[1] > 1 ? 1 : h[1]);
    if (!(n_wi > 0 && n_wo > 0)) return 0.0;
    double a2 = a * a;
    double den = (a2 - 1.0) * nh * nh + 1.0;
    den = PI * den * den;
    double D = a2 / (den + (double)EPS32);
    double g1i = 2.0 * n_wi / (n_wi + sqrt(a2 + (1 - a2) * (n_wi * n_wi)));
    double g1o = 2.0 * n_wo / (n_wo + sqrt(a2 + (1 - a2) * (n_wo * n_wo)));
    double F = schlick(f0, wih);
    double spec = (D * (g1i * g1o) * F) / (4.0 * n_wi * n_wo + (double)EPS32);
    return (double)(float)spec;
}

/* adjoint (extension): d ln(ggx)/d(alpha^2) of the same vectors, alpha^2 = roughness^4 */
static double ggx_dlog_da2(double rough, const double wi_in[3], const double wo_in[3]) {
    double wn = norm3(wi_in[0], wi_in[1], wi_in[2]);
    double wi[3] = {wi_in[0] / wn, wi_in[1] / wn, wi_in[2] / wn};
    double on = norm3(wo_in[0], wo_in[1], wo_in[2]);
    double wo[3] = {wo_in[0] / on, wo_in[1] / on, wo_in[2] / on};
    double h[3] = {wi[0] + wo[0], wi[1] + wo[1], wi[2] + wo[2]};
    double hn = norm3(h[0], h[1], h[2]);
    if (hn == 0.0) hn = 1.0;
    for (int i = 0; i < 3; ++i) h[i] /= hn;
    double a = rough * rough, a2 = a * a;
    double n_wi = wi[1] < 0 ? 0 : (wi[1] > 1 ? 1 : wi[1]);
    double n_wo = wo[1] < 0 ? 0 : (wo[1] > 1 ? 1 : wo[1]);
    double nh = h[1] < 0 ? 0 : (h[1] > 1 ? 1 : h[1]);
    if (!(n_wi > 0 && n_wo > 0)) return 0.0;
    double den = (a2 - 1.0) * nh * nh + 1.0;
    double pd2 = PI * den * den; /* D = a2 / (pd2 + eps): the epsilon's share of the denominator */
    double si = sqrt(a2 + (1 - a2) * (n_wi * n_wi)), so = sqrt(a2 + (1 - a2) * (n_wo * n_wo));
    return 1.0 / a2 - 2.0 * nh * nh / den * (pd2 / (pd2 + (double)EPS32)) - (1.0 - n_wi * n_wi) / (2.0 * si * (n_wi + si)) -
           (1.0 - n_wo * n_wo) / (2.0 * so * (n_wo + so));
}

/* the map directions are float32 and normalised in float32; the view is float64 */
static long long scatter_bin(const AlbLayer* L, const float pd_in[3], const double view_in[3]);
static double scatter_bin_energy(const AlbLayer* L, const float pd_in[3], const double view_in[3]) {
    return L->scatter_weight[scatter_bin(L, pd_in, view_in)];
}
static long long scatter_bin(const AlbLayer* L, const float pd_in[3], const double view_in[3]) {
    volatile float pq = (pd_in[0] * pd_in[0] + pd_in[1] * pd_in[1]) + pd_in[2] * pd_in[2];
    float pn = sqrtf(pq);
    float pd[3] = {pd_in[0] / pn, pd_in[1] / pn, pd_in[2] / pn};
    double vn = norm3(view_in[0], view_in[1], view_in[2]);
    double v[3] = {view_in[0] / vn, view_in[1] / vn, view_in[2] / vn};
    double c = ((double)pd[0] * v[0] + (double)pd[1] * v[1]) + (double)pd[2] * v[2];
    c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
    double th = acos(c);
    double width = L->bin_width;
    long long i = (long long)((th - (double)EPS32) / width);
    if (i < 0) i = 0;
    if (i > NDIV - 1) i = NDIV - 1;
    return i;
}

/* Gather queries of one kind against one map and add into waveform[nbins] (float64).
 * map: pos float[3m], dir float[3m], energy/time float[m], fwi/sfi float[3m] (nullable);
 * queries: pos/dir double[3q], energy/time float[q]. rk_out (nullable) gets r_k per query.
 * heat_w/heat_f (nullable, bins*bins) receive the sampled heatmaps.
 * Adjoint (extension): with mscore/qscore (float[4m] / float[4q]: a, b, g, albedo) and jac
 * (float64 [5][nbins]: a, b, g, albedo, roughness) non-null, every neighbour adds
 * c (s_query + s_record + d ln w/d theta) to jac. */
int oracle_gather(const AlbSceneParams* p, int channel, const float* mpos, const float* mdir, const float* menergy,
                  const float* mtime, const float* mfwi, const float* msfi, int64_t m, const double* qpos,
                  const double* qdir, const float* qenergy, const float* qtime, int64_t nq, double* waveform,
                  double* rk_out, double* heat_w, double* heat_f, const float* mscore, const float* qscore,
                  double* jac, int threads) {
    const int nj = (mscore && qscore && jac) ? 5 : 0;
    int k = p->k;
    /* extension: a gated window keeps bins [gate_start, gate_start + gate_bins) only */
    const int gated = p->gate_bins > 0;
    int64_t nb = gated ? p->gate_bins : 2 * p->steps;
    const double R = p->gather_radius;  /* extension: > 0 selects the fixed-radius gather */
    if (nq > 0 && R <= 0.0 && m < k) return ALB_ERR_TOO_FEW;
    int nthreads = 1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
    nthreads = omp_get_max_threads();
#endif
    int hb = p->heatmap_enabled ? p->heatmap_bins * p->heatmap_bins : 0;
    const size_t stride = (size_t)nb + 2 * hb + (size_t)nj * nb;
    double* priv = (double*)calloc((size_t)nthreads * stride, sizeof(double));
    int err = 0;
    KdTree* tree = (g_knn_brute || nq == 0 || m == 0) ? NULL : kd_build(mpos, m);
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* wf = priv + (size_t)tid * stride;
        double* hw = wf + nb;
        double* hf = hw + hb;
        double* jp = hf + hb;
        int64_t ccap = R > 0.0 ? 64 : k;
        Cand* c = (Cand*)malloc((size_t)ccap * sizeof(Cand));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 8)
#endif
        for (int64_t q = 0; q < nq; ++q) {
            const double* x = qpos + 3 * q;
            const double* ds = qdir + 3 * q;
            int64_t cnt = k;
            double r;
            if (R > 0.0) {
                /* every record with float64 squared distance <= R^2 */
                cnt = 0;
                if (tree) {
                    kd_range_node(tree, mpos, 0, x, R * R, &c, &cnt, &ccap);
                    qsort(c, (size_t)cnt, sizeof(Cand), cand_idx_cmp);
                }
                for (int64_t j = 0; j < m && !tree; ++j) {
                    double dx = (double)mpos[3 * j] - x[0], dy = (double)mpos[3 * j + 1] - x[1],
                           dz = (double)mpos[3 * j + 2] - x[2];
                    if ((dx * dx + dy * dy) + dz * dz <= R * R) {
                        if (cnt == ccap) {
                            ccap *= 2;
                            c = (Cand*)realloc(c, (size_t)ccap * sizeof(Cand));
                        }
                        c[cnt].i = (int32_t)j;
                        ++cnt;
                    }
                }
                r = R;
            } else {
                if (tree) knn_tree(tree, mpos, x, k, c);
                else knn_brute(mpos, m, x, k, c);
                r = sqrt(c[k - 1].d2);
            }
            if (rk_out) rk_out[q] = r;
            double ks = (channel == ALB_SCATTER) ? (4.0 / 3.0) * PI * pow(r, 3.0) : PI * (r * r);
            double norm = 1.0 / ks;
            double view[3] = {-ds[0], -ds[1], -ds[2]};
            int L = 0;
            if (channel == ALB_SCATTER) {
                double depth = -(x[1] - p->surface_y);
                while (L < p->n_layers && !(p->layers[L].bottom_depth > depth)) ++L;
                if (L >= p->n_layers) L = p->n_layers - 1;
            }
            for (int64_t j = 0; j < cnt; ++j) {
                int32_t id = c[j].i;
                double w;
                const float* df = mdir + 3 * id;
                if (channel == ALB_BOTTOM_REFLECTION) {
                    double ct = -ds[1];
                    w = (p->seafloor_albedo / PI) * (ct > 0.0 ? ct : 0.0);
                } else if (channel == ALB_SURFACE_TRANSMISSION_UP) {
                    w = p->surface_albedo / PI;
                } else if (channel == ALB_SCATTER) {
                    w = scatter_bin_energy(&p->layers[L], df, view);
                } else {
                    double wi[3] = {-(double)df[0], -(double)df[1], -(double)df[2]};
                    w = ggx(p->roughness, p->f0, wi, view);
                }
                float e32 = qenergy[q] * menergy[id];
                double contrib = ((double)e32 * norm) * w;
                float tsum = qtime[q] + mtime[id];
                long long bin = (long long)(tsum / (float)p->sample_multiplier) - (gated ? p->gate_start : 0);
                const int in_window = bin >= 0 && bin < nb;
                if (!in_window && !gated) {
                    err = ALB_ERR_CAPACITY;
                    continue;
                }
                if (in_window) wf[bin] += contrib;
                if (nj && in_window) {
                    const float* sq = qscore + 4 * q;
                    const float* sp = mscore + 4 * (int64_t)id;
                    double d[5] = {(double)sq[0] + sp[0], (double)sq[1] + sp[1], (double)sq[2] + sp[2],
                                   (double)sq[3] + sp[3], 0.0};
                    if (channel == ALB_SCATTER && p->layers[L].dlog_weight_g)
                        d[2] += p->layers[L].dlog_weight_g[scatter_bin(&p->layers[L], df, view)];
                    if (channel == ALB_BOTTOM_REFLECTION && p->seafloor_albedo > 0.0) d[3] += 1.0 / p->seafloor_albedo;
                    if (channel == ALB_SURFACE_REFLECTION) {
                        double wi[3] = {-(double)df[0], -(double)df[1], -(double)df[2]};
                        double r = p->roughness;
                        d[4] = 4.0 * r * r * r * ggx_dlog_da2(r, wi, view);
                    }
                    for (int t = 0; t < 5; ++t) jp[(int64_t)t * nb + bin] += contrib * d[t];
                }
                if (hb && mfwi) {
                    const float* fw = mfwi + 3 * id;
                    const float* sf = msfi + 3 * id;
                    double wb = 2.0 * p->heatmap_water_extent / p->heatmap_bins;
                    double fb = 2.0 * p->heatmap_floor_extent / p->heatmap_bins;
                    if (!isnan(fw[0])) {
                        long long xi = (long long)(((double)fw[0] - p->water_center[0] + p->heatmap_water_extent) / wb);
                        long long zi = (long long)(((double)fw[2] - p->water_center[2] + p->heatmap_water_extent) / wb);
                        if (xi >= 0 && xi < p->heatmap_bins && zi >= 0 && zi < p->heatmap_bins)
                            hw[xi * p->heatmap_bins + zi] += contrib;
                    }
                    if (!isnan(sf[0])) {
                        long long xi = (long long)(((double)sf[0] - p->floor_center[0] + p->heatmap_floor_extent) / fb);
                        long long zi = (long long)(((double)sf[2] - p->floor_center[2] + p->heatmap_floor_extent) / fb);
                        if (xi >= 0 && xi < p->heatmap_bins && zi >= 0 && zi < p->heatmap_bins)
                            hf[xi * p->heatmap_bins + zi] += contrib;
                    }
                }
            }
        }
        free(c);
    }
    for (int t = 0; t < nthreads; ++t) {
        const double* wf = priv + (size_t)t * stride;
        for (int64_t b = 0; b < nb; ++b) waveform[b] += wf[b];
        for (int64_t b = 0; b < (int64_t)nj * nb; ++b) jac[b] += wf[nb + 2 * hb + b];
        if (hb && heat_w)
            for (int b = 0; b < hb; ++b) {
                heat_w[b] += wf[nb + b];
                heat_f[b] += wf[nb + hb + b];
            }
    }
    free(priv);
    kd_free(tree);
    return err;
}

/* ------------------------------------------------------------------------------------ */
/* exported: single-function hooks for known-answer tests                               */
/* ------------------------------------------------------------------------------------ */

/* microfacet_reflected_energy(wi[n], wo, +y, roughness, f0) -> out[n] */
void oracle_ggx_batch(double roughness, double f0, const double* wi, int64_t n, const double* wo, double* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = ggx(roughness, f0, wi + 3 * i, wo);
}

/* calculate_energy_batch(pdirs float32[n], view) with the layer's tables -> out[n] */
void oracle_scatter_energy_batch(const AlbSceneParams* p, int layer, const float* pdirs, int64_t n,
                                 const double* view, double* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = scatter_bin_energy(&p->layers[layer], pdirs + 3 * i, view);
}

/* sizeof / offsetof of the ABI structs, to check the Python ctypes mirror */
#include <stddef.h>
void oracle_abi_layout(int64_t* out) {
    out[0] = (int64_t)sizeof(AlbSceneParams);
    out[1] = (int64_t)sizeof(AlbLayer);
    out[2] = (int64_t)offsetof(AlbSceneParams, layers);
    out[3] = (int64_t)offsetof(AlbSceneParams, water_center);
    out[4] = (int64_t)offsetof(AlbSceneParams, laser_rot);
    out[5] = (int64_t)offsetof(AlbLayer, phase_theta);
    out[6] = (int64_t)sizeof(AlbReplay);
}
