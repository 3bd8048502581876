// C ABI of the GB300 photon-tracing / photon-mapping engine (declared in include/albgpu.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "albgpu.h"
#include "internal.h"
#include "tracer_fast.cuh"

using namespace alb;

#include <atomic>
static std::atomic<long long> g_launches{0};
namespace alb {
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long launches_total() { return g_launches.load(); }
}  // namespace alb

// ------------------------------------------------------------------------------------------
// Workspace
// ------------------------------------------------------------------------------------------

Workspace::~Workspace() {
    for (void* p : temps_) cudaFree(p);
    if (box_) cudaFree(box_);
}

void* Workspace::take_bytes(uint64_t bytes) {
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    if (cudaMallocAsync(&p, bytes, st_) != cudaSuccess) {
        failed_ = true;
        cudaGetLastError();
        return nullptr;
    }
    temps_.push_back(p);
    return p;
}

void Workspace::release(size_t m) {
    while (temps_.size() > m) {
        cudaFreeAsync(temps_.back(), st_);
        temps_.pop_back();
    }
}

unsigned* Workspace::scratch_box() {
    if (!box_) {
        if (cudaMalloc(&box_, 64 * sizeof(unsigned)) != cudaSuccess) {
            failed_ = true;
            cudaGetLastError();
        }
    }
    return box_;
}

static void* grow(void* old, uint64_t& cap, uint64_t n, size_t elem, bool& failed) {
    if (cap >= n && old) return old;
    if (old) {
        cudaDeviceSynchronize();
        cudaFree(old);
    }
    uint64_t want = std::max<uint64_t>(n + n / 32, 256);
    void* p = nullptr;
    if (cudaMalloc(&p, want * elem) != cudaSuccess) {
        cudaGetLastError();
        failed = true;
        cap = 0;
        return nullptr;
    }
    cap = want;
    return p;
}

void* Workspace::alloc_persistent(void* old, uint64_t& cap, uint64_t n) { return grow(old, cap, n, 16, failed_); }
void* Workspace::alloc_persistent_u32(void* old, uint64_t& cap, uint64_t n) { return grow(old, cap, n, 4, failed_); }

// ------------------------------------------------------------------------------------------
// Context
// ------------------------------------------------------------------------------------------

struct AlbCtx {
    int device = 0;
    cudaStream_t st = 0;
    SceneDev sc{};
    FastScene fast{};
    std::vector<void*> tables;
    Workspace ws;
    // forward records
    RecordStore rec[ALB_CHANNELS];
    uint64_t rec_id_cap[ALB_CHANNELS] = {0};
    uint64_t fwi_cap[ALB_CHANNELS] = {0}, sfi_cap[ALB_CHANNELS] = {0}, b_cap[ALB_CHANNELS] = {0};
    unsigned long long* d_rec_count = nullptr;
    uint64_t h_rec_count[ALB_CHANNELS] = {0};
    double rec_rate[ALB_CHANNELS] = {2.0, 8.0, 1.05, 1.05};
    MapIndex map[ALB_CHANNELS];
    bool maps_built = false;
    // records of a channel live either in its append store or, once indexed, only in the
    // index (the store is released to make room; restored if more records are appended)
    bool rec_released[ALB_CHANNELS] = {false, false, false, false};
    // backward queries
    float4* qa[3] = {nullptr, nullptr, nullptr};
    float4* qb[3] = {nullptr, nullptr, nullptr};
    float4* qc[3] = {nullptr, nullptr, nullptr};
    uint32_t* qid[3] = {nullptr, nullptr, nullptr};
    float4* qs[3] = {nullptr, nullptr, nullptr};  // adjoint query scores
    uint32_t* qperm[3] = {nullptr, nullptr, nullptr};
    double* qrk[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    uint64_t qcap[3] = {0, 0, 0}, qcap_b[3] = {0}, qcap_c[3] = {0}, qid_cap[3] = {0}, qperm_cap[3] = {0};
    uint64_t qrk_cap[3][2] = {{0}};
    unsigned long long* d_q_count = nullptr;
    uint64_t h_q_count[3] = {0, 0, 0};
    double q_rate[3] = {2.0, 8.0, 1.05};
    // accumulators
    unsigned long long* wf = nullptr;  // lo words then hi words, [2][channels][nbins]
    unsigned long long* hm = nullptr;  // sampled heatmaps, [2 maps][2 words][bins*bins]
    unsigned* hm_radius = nullptr;
    // adjoint Jacobian: lo words then hi words, [2][kJacParams][channels][nbins]
    unsigned long long* jac = nullptr;
    int64_t wf_bins = 0, jac_bins = 0, hm_cells = 0, hm_radius_cells = 0;  // accumulator capacities
    // per-layer scene tables (device), reused when the context takes a new scene
    struct LayerTables {
        void *th = nullptr, *cdf = nullptr, *sl = nullptr, *w = nullptr, *dlw = nullptr, *dsg = nullptr, *inv = nullptr;
    } lt[ALB_MAX_LAYERS];
    bool keep_records = false;  // keep the append stores after indexing (batched runs)
    // exit states
    double* ex_pos = nullptr;
    double* ex_dir = nullptr;
    float* ex_f = nullptr;
    uint64_t ex_cap = 0, ex_n = 0;
    // misc
    int* d_err = nullptr;
    unsigned long long* d_stats = nullptr;
    int keep_exit = 0, keep_ids = 0, precise = 1, sort_q = 1;
    int64_t map_cap_hint = 0;
    int launches = 0;
    std::string err;
    // phase timing (CUDA events on the context's stream)
    double phase_ms[ALB_PHASES] = {0};
    int64_t phase_calls[ALB_PHASES] = {0};
    int64_t gathered[ALB_CHANNELS] = {0};
    cudaEvent_t ev[2 * ALB_PHASES] = {};
    bool ev_ready = false;
};

// Time one phase: record a start event, run `body`, record a stop event, and fold the
// elapsed time into the accumulator once the stream has drained (the caller syncs).
struct PhaseTimer {
    AlbCtx* c;
    int phase;
    PhaseTimer(AlbCtx* ctx, int p) : c(ctx), phase(p) {
        if (!c->ev_ready) {
            for (auto& e : c->ev) cudaEventCreate(&e);
            c->ev_ready = true;
        }
        cudaEventRecord(c->ev[2 * phase], c->st);
    }
    void stop() {
        cudaEventRecord(c->ev[2 * phase + 1], c->st);
        cudaEventSynchronize(c->ev[2 * phase + 1]);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev[2 * phase], c->ev[2 * phase + 1]) == cudaSuccess) c->phase_ms[phase] += ms;
        c->phase_calls[phase] += 1;
    }
};

static int fail(AlbCtx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(ctx, ALB_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

static int check_device(AlbCtx* ctx, const char* where) {
    cudaError_t e = cudaStreamSynchronize(ctx->st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, ALB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    if (ctx->ws.failed()) {
        ctx->ws.clear_failed();
        return fail(ctx, ALB_ERR_CUDA, std::string(where) + ": device allocation failed");
    }
    int h = 0;
    CK(cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (h != 0) {
        CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        const char* what = h == ALB_ERR_ITER_CAP ? "a device loop hit its iteration cap"
                           : h == ALB_ERR_REPLAY ? "a replay stream ran out of variates"
                           : h == ALB_ERR_TOO_FEW ? "a photon map holds fewer records than k"
                           : h == ALB_ERR_CAPACITY ? "a waveform bin index fell outside the waveform"
                           : h == ALB_ERR_INVALID ? "a neighbour search admitted fewer than k finite points "
                                                    "(NaN or infinite coordinates)"
                                                   : "device error";
        return fail(ctx, h, std::string(where) + ": " + what);
    }
    return ALB_OK;
}

static thread_local std::string g_create_error;

namespace alb {
// message of a failure that has no context (alb_create, alb_knn_noalloc)
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace alb

extern "C" const char* alb_last_error(const AlbCtx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

static void* table_buf(void*& slot, size_t bytes) {
    if (!slot && cudaMalloc(&slot, bytes) != cudaSuccess) {
        cudaGetLastError();
        slot = nullptr;
    }
    return slot;
}

// Scene constants and tables of p into ctx->sc. The per-layer table buffers belong to the
// context and are reused by a later scene (batched runs re-scene one context per stream);
// copies are ordered on the context's stream, drained before the host staging vectors go
// away. Returns "" or why the scene is invalid.
static std::string set_scene(AlbCtx* ctx, const AlbSceneParams* p) {
    if (!(p->dt > 0) || p->steps <= 0 || p->sample_multiplier <= 0) return std::string("bad time step");
    if (p->k < 1 || p->k > 256) return std::string("photon_mapping_k must be in [1, 256]");
    if (p->n_layers < 1 || p->n_layers > ALB_MAX_LAYERS) return std::string("1..8 water layers supported");
    if (!(p->surface_y > p->floor_y)) return std::string("seafloor must lie below the surface");
    const int32_t adjoint = ctx->sc.adjoint;
    if (adjoint)
        for (int l = 0; l < p->n_layers; ++l)
            if (p->layers[l].profiled) return std::string("the adjoint needs constant layers");
    SceneDev& s = ctx->sc;
    s.dt = p->dt;
    s.total_steps = p->steps * (int64_t)p->sample_multiplier;
    s.nbins = 2 * p->steps;
    s.gate_lo = 0;
    s.gated = 0;
    if (p->gate_bins < 0 || p->gate_start < 0) return std::string("gate_start and gate_bins must be >= 0");
    s.stop_step[ALB_FORWARD] = s.stop_step[ALB_BACKWARD] = s.total_steps;
    if (p->gate_bins > 0) {
        if (p->gate_start + p->gate_bins > 2 * p->steps) return std::string("the gate must lie inside the timeline");
        s.nbins = p->gate_bins;
        s.gate_lo = p->gate_start;
        s.gated = 1;
        // With the fixed-radius gather every (query, record) pair contributes on its own. A
        // contribution lands in bin (t_query + t_record) / multiplier. Every photon starts at
        // the origin, |surface_y| above the water, and no record or query is made before it
        // reaches the surface: t >= floor(|surface_y| / (c_air dt)) - 2 steps, less the
        // forward pulse offset (bounded by 7 sigma / effective rate steps). A photon of one
        // pass can therefore stop once its steps exceed the gate's end minus the other
        // pass's earliest time: nothing it would add later can land in the window. (The
        // k-NN estimate is not pairwise: a late record can still be among a query's k
        // nearest and set its radius, so k-NN runs trace the whole timeline.)
        const double step_air = p->speed_air * p->dt;
        const int64_t t_surface = std::max<int64_t>((int64_t)std::floor(-p->surface_y / step_air) - 2, 0);
        const int64_t pulse = (int64_t)std::ceil(7.0 * p->pulse_sigma / (double)(float)p->effective_rate) + 1;
        const int64_t end = (p->gate_start + p->gate_bins + 2) * (int64_t)p->sample_multiplier;
        const int64_t fwd = end - t_surface + pulse + 4;                           // queries start >= t_surface
        const int64_t bwd = end - std::max<int64_t>(t_surface - pulse, 0) + 4;     // records start >= t_surface - pulse
        if (p->gather_radius > 0.0) {
            s.stop_step[ALB_FORWARD] = std::min(s.total_steps, std::max<int64_t>(fwd, 0));
            s.stop_step[ALB_BACKWARD] = std::min(s.total_steps, std::max<int64_t>(bwd, 0));
        }
    }
    s.mult = p->sample_multiplier;
    s.k = p->k;
    s.ys = p->surface_y;
    s.yf = p->floor_y;
    s.v_air = p->speed_air;
    s.n_water = p->n_water;
    s.eta = 1.0 / p->n_water;
    s.f0 = p->f0;
    s.floor_albedo = p->seafloor_albedo;
    s.floor_albedo32 = (float)p->seafloor_albedo;
    s.surface_albedo = p->surface_albedo;
    s.roughness = p->roughness;
    double ga = p->roughness * p->roughness;
    s.ggx_a2 = (float)(ga * ga);
    for (int i = 0; i < 9; ++i) s.rot_d[i] = (double)p->laser_rot[i];
    s.div = p->divergence;
    s.fov = p->fov;
    s.cos_fov = std::cos(p->fov);
    s.aperture = p->aperture_radius;
    s.pulse_sigma32 = p->pulse_sigma;
    s.eff_rate32 = (double)(float)p->effective_rate;
    s.rayleigh_sigma = p->divergence / 3.0;
    s.rayleigh_mass = -std::expm1(-(p->divergence * p->divergence) / (2.0 * s.rayleigh_sigma * s.rayleigh_sigma));
    s.n_layers = p->n_layers;
    if (!(p->gather_radius >= 0.0)) return std::string("gather_radius must be >= 0 (0 selects the k-NN gather)");
    if (!(p->slope_sigma >= 0.0)) return std::string("slope_sigma must be >= 0");
    s.slope_sigma = p->slope_sigma;
    s.radius = p->gather_radius;
    s.heatmap = p->heatmap_enabled;
    s.hm_bins = p->heatmap_bins;
    s.hm_wext = p->heatmap_water_extent;
    s.hm_fext = p->heatmap_floor_extent;
    s.hm_wbin = 2.0 * p->heatmap_water_extent / p->heatmap_bins;
    s.hm_fbin = 2.0 * p->heatmap_floor_extent / p->heatmap_bins;
    for (int i = 0; i < 3; ++i) {
        s.wc[i] = p->water_center[i];
        s.fc[i] = p->floor_center[i];
    }
    s.adjoint = adjoint;
    s.inv_albedo = p->seafloor_albedo > 0.0 ? (float)(1.0 / p->seafloor_albedo) : 0.f;
    s.dla2_drough = (float)(4.0 * p->roughness * p->roughness * p->roughness);
    const int N = ALB_PHASE_DIVISIONS;
    for (int l = 0; l < p->n_layers; ++l) {
        const AlbLayer& L = p->layers[l];
        if (!L.phase_theta || !L.phase_cdf || !L.phase_slope || !L.scatter_weight) return std::string("missing layer table");
        for (int i = 0; i < 3; ++i) {
            s.adj_dla[l][i] = (float)L.dlog_alpha[i];
            s.adj_dls[l][i] = (float)L.dlog_ssa[i];
        }
        s.layer_hg_g[l] = (float)L.hg_g;
        s.layer_dlw_g[l] = nullptr;
        if (L.dlog_weight_g) {
            std::vector<float> d(N);
            for (int i = 0; i < N; ++i) d[i] = (float)L.dlog_weight_g[i];
            float* dd = (float*)table_buf(ctx->lt[l].dlw, N * sizeof(float));
            if (!dd) return std::string("table allocation failed");
            cudaMemcpyAsync(dd, d.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx->st);
            cudaStreamSynchronize(ctx->st);
            s.layer_dlw_g[l] = dd;
        }
        s.layer_dsg[l] = nullptr;
        if (L.dlog_sample_g) {
            std::vector<float> d(N);
            for (int i = 0; i < N; ++i) d[i] = (float)L.dlog_sample_g[i];
            float* dd = (float*)table_buf(ctx->lt[l].dsg, N * sizeof(float));
            if (!dd) return std::string("table allocation failed");
            cudaMemcpyAsync(dd, d.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx->st);
            cudaStreamSynchronize(ctx->st);
            s.layer_dsg[l] = dd;
        }
        s.layer_bottom[l] = L.bottom_depth;
        s.layer_speed[l] = L.speed;
        s.layer_alpha[l] = L.alpha;
        s.layer_ssa[l] = L.ssa;
        s.layer_binw[l] = (float)L.bin_width;
        s.layer_h[l] = L.height;
        s.layer_top32[l] = L.top32;
        s.layer_prof[l] = L.profiled ? 1 : 0;
        s.layer_lut_n[l] = 0;
        s.layer_lut_z[l] = nullptr;
        s.layer_lut_a[l] = nullptr;
        s.layer_nkind[l] = s.layer_akind[l] = 0;
        s.layer_n0[l] = s.layer_n1[l] = s.layer_a0[l] = s.layer_a1[l] = 0.0;
        if (L.profiled) {
            if (!L.lut_z || !L.lut_alpha || L.lut_n < 2) return std::string("profiled layer without an attenuation table");
            if (!(L.height > 0.0)) return std::string("profiled layer needs a positive height");
            if (L.n_kind < 0 || L.n_kind > 2 || L.a_kind < 0 || L.a_kind > 2) return std::string("unknown profile kind");
            float* lz;
            double* la;
            if (cudaMalloc(&lz, L.lut_n * sizeof(float)) != cudaSuccess ||
                cudaMalloc(&la, L.lut_n * sizeof(double)) != cudaSuccess)
                return std::string("table allocation failed");
            ctx->tables.insert(ctx->tables.end(), {lz, la});
            cudaMemcpyAsync(lz, L.lut_z, L.lut_n * sizeof(float), cudaMemcpyHostToDevice, ctx->st);
            cudaMemcpyAsync(la, L.lut_alpha, L.lut_n * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
            s.layer_lut_n[l] = L.lut_n;
            s.layer_lut_z[l] = lz;
            s.layer_lut_a[l] = la;
            s.layer_nkind[l] = L.n_kind;
            s.layer_akind[l] = L.a_kind;
            s.layer_n0[l] = L.n_start;
            s.layer_n1[l] = L.n_end;
            s.layer_a0[l] = L.a_start;
            s.layer_a1[l] = L.a_end;
        }
        double* th = (double*)table_buf(ctx->lt[l].th, N * sizeof(double));
        double* cdf = (double*)table_buf(ctx->lt[l].cdf, N * sizeof(double));
        double* sl = (double*)table_buf(ctx->lt[l].sl, N * sizeof(double));
        float* w = (float*)table_buf(ctx->lt[l].w, N * sizeof(float));
        if (!th || !cdf || !sl || !w) return std::string("table allocation failed");
        std::vector<double> slope(N, 0.0);
        std::memcpy(slope.data(), L.phase_slope, (N - 1) * sizeof(double));
        std::vector<float> wf(N);
        for (int i = 0; i < N; ++i) wf[i] = (float)L.scatter_weight[i];
        cudaMemcpyAsync(th, L.phase_theta, N * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
        cudaMemcpyAsync(cdf, L.phase_cdf, N * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
        cudaMemcpyAsync(sl, slope.data(), N * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
        cudaMemcpyAsync(w, wf.data(), N * sizeof(float), cudaMemcpyHostToDevice, ctx->st);
        s.layer_theta[l] = th;
        s.layer_cdf[l] = cdf;
        s.layer_slope[l] = sl;
        s.layer_weight[l] = w;
        // inverse CDF theta(u) at u = j / kInvCdf for the fast tracer (numpy.interp restated)
        std::vector<float> inv(kInvCdf + 1);
        for (int j = 0; j <= kInvCdf; ++j) {
            double u = (double)j / kInvCdf;
            double t;
            if (u < L.phase_cdf[0]) t = L.phase_theta[0];
            else if (u >= L.phase_cdf[N - 1]) t = L.phase_theta[N - 1];
            else {
                int lo = 0, hi = N - 1;
                while (hi - lo > 1) {
                    int mid = (lo + hi) / 2;
                    if (L.phase_cdf[mid] <= u) lo = mid; else hi = mid;
                }
                t = (u == L.phase_cdf[lo]) ? L.phase_theta[lo] : L.phase_slope[lo] * (u - L.phase_cdf[lo]) + L.phase_theta[lo];
            }
            inv[j] = (float)t;
        }
        float* dinv = (float*)table_buf(ctx->lt[l].inv, (kInvCdf + 1) * sizeof(float));
        if (!dinv) return std::string("table allocation failed");
        cudaMemcpyAsync(dinv, inv.data(), (kInvCdf + 1) * sizeof(float), cudaMemcpyHostToDevice, ctx->st);
        cudaStreamSynchronize(ctx->st);  // the host staging vectors die with this iteration
        ctx->fast.inv_theta[l] = dinv;
    }
    return std::string();
}

// Waveform, Jacobian and heatmap accumulators sized for the current scene (grown, never
// shrunk; a grown buffer is zeroed by the next reset).
static std::string ensure_accumulators(AlbCtx* ctx) {
    const SceneDev& s = ctx->sc;
    auto regrow = [&](unsigned long long*& buf, int64_t& have, int64_t need, size_t words_per) -> bool {
        if (buf && have >= need) return true;
        if (buf) {
            cudaStreamSynchronize(ctx->st);
            cudaFree(buf);
            buf = nullptr;
        }
        if (cudaMalloc(&buf, (size_t)need * words_per * 8) != cudaSuccess) {
            cudaGetLastError();
            buf = nullptr;
            have = 0;
            return false;
        }
        cudaMemsetAsync(buf, 0, (size_t)need * words_per * 8, ctx->st);
        have = need;
        return true;
    };
    if (!regrow(ctx->wf, ctx->wf_bins, s.nbins, (size_t)2 * ALB_CHANNELS)) return "waveform allocation failed";
    if (s.adjoint && !regrow(ctx->jac, ctx->jac_bins, s.nbins, (size_t)2 * kJacParams * ALB_CHANNELS))
        return "jacobian allocation failed";
    if (s.heatmap) {
        const int64_t hb = (int64_t)s.hm_bins * s.hm_bins;
        if (!regrow(ctx->hm, ctx->hm_cells, hb, 4)) return "heatmap allocation failed";
        if (!ctx->hm_radius || ctx->hm_radius_cells < hb) {
            if (ctx->hm_radius) {
                cudaStreamSynchronize(ctx->st);
                cudaFree(ctx->hm_radius);
            }
            if (cudaMalloc(&ctx->hm_radius, hb * 4) != cudaSuccess) {
                ctx->hm_radius = nullptr;
                return "heatmap allocation failed";
            }
            cudaMemsetAsync(ctx->hm_radius, 0, hb * 4, ctx->st);
            ctx->hm_radius_cells = hb;
        }
    }
    return std::string();
}

extern "C" int alb_create(const AlbSceneParams* p, int device, AlbCtx** out) {
    if (!p || !out) return ALB_ERR_INVALID;
    *out = nullptr;
    AlbCtx* ctx = new AlbCtx();
    auto bad = [&](const std::string& m) {
        g_create_error = m;
        alb_destroy(ctx);
        return ALB_ERR_INVALID;
    };
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) return bad("cudaSetDevice failed");
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    std::string e = set_scene(ctx, p);
    if (e.empty()) e = ensure_accumulators(ctx);
    if (!e.empty()) return bad(e);
    if (cudaMalloc(&ctx->d_rec_count, ALB_CHANNELS * 8) != cudaSuccess || cudaMalloc(&ctx->d_q_count, 3 * 8) != cudaSuccess ||
        cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess || cudaMalloc(&ctx->d_stats, 32 * 8) != cudaSuccess)
        return bad("counter allocation failed");
    cudaMemset(ctx->d_rec_count, 0, ALB_CHANNELS * 8);
    cudaMemset(ctx->d_q_count, 0, 3 * 8);
    cudaMemset(ctx->d_err, 0, sizeof(int));
    cudaMemset(ctx->d_stats, 0, 32 * 8);
    if (cudaDeviceSynchronize() != cudaSuccess) return bad("device initialisation failed");
    *out = ctx;
    return ALB_OK;
}

extern "C" void alb_destroy(AlbCtx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (void* p : ctx->tables) cudaFree(p);
    for (int c = 0; c < ALB_CHANNELS; ++c) {
        cudaFree(ctx->rec[c].a); cudaFree(ctx->rec[c].fwi); cudaFree(ctx->rec[c].sfi);
        cudaFree(ctx->rec[c].id); cudaFree(ctx->rec[c].sco);
        MapIndex& m = ctx->map[c];
        cudaFree(m.a); cudaFree(m.b); cudaFree(m.fwi); cudaFree(m.sfi); cudaFree(m.id); cudaFree(m.sco);
        cudaFree(m.box_lo); cudaFree(m.box_hi);
    }
    for (int k = 0; k < 3; ++k) {
        cudaFree(ctx->qa[k]); cudaFree(ctx->qb[k]); cudaFree(ctx->qc[k]); cudaFree(ctx->qid[k]); cudaFree(ctx->qperm[k]);
        cudaFree(ctx->qrk[k][0]); cudaFree(ctx->qrk[k][1]); cudaFree(ctx->qs[k]);
    }
    cudaFree(ctx->wf); cudaFree(ctx->hm); cudaFree(ctx->hm_radius); cudaFree(ctx->jac);
    for (auto& t : ctx->lt) {
        cudaFree(t.th); cudaFree(t.cdf); cudaFree(t.sl); cudaFree(t.w); cudaFree(t.dlw); cudaFree(t.dsg); cudaFree(t.inv);
    }
    cudaFree(ctx->ex_pos); cudaFree(ctx->ex_dir); cudaFree(ctx->ex_f);
    cudaFree(ctx->d_rec_count); cudaFree(ctx->d_q_count); cudaFree(ctx->d_err); cudaFree(ctx->d_stats);
    if (ctx->ev_ready)
        for (auto& e : ctx->ev) cudaEventDestroy(e);
    delete ctx;
}

extern "C" int alb_set_option(AlbCtx* ctx, int key, int64_t v) {
    if (!ctx) return ALB_ERR_INVALID;
    switch (key) {
        case ALB_OPT_KEEP_EXIT_STATES: ctx->keep_exit = (int)v; break;
        case ALB_OPT_KEEP_RECORD_IDS: ctx->keep_ids = (int)v; break;
        case ALB_OPT_PRECISE: ctx->precise = (int)v; break;
        case ALB_OPT_MAP_CAPACITY: ctx->map_cap_hint = v; break;
        case ALB_OPT_SORT_QUERIES: ctx->sort_q = (int)v; break;
        case ALB_OPT_STREAM:
            ctx->st = (cudaStream_t)(intptr_t)v;
            ctx->ws.set_stream(ctx->st);
            break;
        case ALB_OPT_ADJOINT: {
            for (int c = 0; c < ALB_CHANNELS; ++c)
                if (ctx->h_rec_count[c]) return fail(ctx, ALB_ERR_STATE, "set ALB_OPT_ADJOINT before the first forward trace");
            if (v) {
                for (int l = 0; l < ctx->sc.n_layers; ++l)
                    if (ctx->sc.layer_prof[l]) return fail(ctx, ALB_ERR_INVALID, "the adjoint needs constant layers");
            }
            ctx->sc.adjoint = v ? 1 : 0;
            if (v) {
                std::string e = ensure_accumulators(ctx);
                if (!e.empty()) return fail(ctx, ALB_ERR_CUDA, e);
                CK(cudaStreamSynchronize(ctx->st));
            }
            break;
        }
        default: return fail(ctx, ALB_ERR_INVALID, "unknown option");
    }
    return ALB_OK;
}

// grow a record store to hold `need` records, preserving the first `keep`
// backward photons traced and gathered per chunk when no per-photon state is exported
constexpr uint64_t kBackwardChunk = 1ull << 22;

static int ensure_records(AlbCtx* ctx, int c, uint64_t need, uint64_t keep) {
    RecordStore& r = ctx->rec[c];
    bool want_hm = ctx->sc.heatmap != 0;
    bool want_id = ctx->keep_ids != 0;
    bool want_sco = ctx->sc.adjoint != 0;
    if (r.cap >= need && (!want_id || r.id) && (!want_hm || r.fwi) && (!want_sco || r.sco)) return ALB_OK;
    uint64_t cap = std::max<uint64_t>(need + need / 16, 1024);
    if (!keep) {  // nothing to copy: release the old store first, so the peak is one store
        CK(cudaStreamSynchronize(ctx->st));
        cudaFree(r.a); cudaFree(r.fwi); cudaFree(r.sfi); cudaFree(r.id); cudaFree(r.sco);
        r = RecordStore{};
    }
    float4 *a = nullptr, *fwi = nullptr, *sfi = nullptr, *sco = nullptr;
    uint32_t* id = nullptr;
    // every allocation is checked, and a failure frees what this call had taken; the two
    // record halves are interleaved in one allocation (RecordStore)
    bool ok = cudaMalloc(&a, cap * 32) == cudaSuccess;
    if (ok && want_hm) ok = cudaMalloc(&fwi, cap * 16) == cudaSuccess && cudaMalloc(&sfi, cap * 16) == cudaSuccess;
    if (ok && want_id) ok = cudaMalloc(&id, cap * 4) == cudaSuccess;
    if (ok && want_sco) ok = cudaMalloc(&sco, cap * 16) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cudaFree(a); cudaFree(fwi); cudaFree(sfi); cudaFree(id); cudaFree(sco);
        return fail(ctx, ALB_ERR_CUDA, "photon-map store: out of device memory");
    }
    if (keep) {
        CK(cudaMemcpyAsync(a, r.a, keep * 32, cudaMemcpyDeviceToDevice, ctx->st));
        if (want_hm && r.fwi) {
            CK(cudaMemcpyAsync(fwi, r.fwi, keep * 16, cudaMemcpyDeviceToDevice, ctx->st));
            CK(cudaMemcpyAsync(sfi, r.sfi, keep * 16, cudaMemcpyDeviceToDevice, ctx->st));
        }
        if (want_id && r.id) CK(cudaMemcpyAsync(id, r.id, keep * 4, cudaMemcpyDeviceToDevice, ctx->st));
        if (want_sco && r.sco) CK(cudaMemcpyAsync(sco, r.sco, keep * 16, cudaMemcpyDeviceToDevice, ctx->st));
    }
    CK(cudaStreamSynchronize(ctx->st));
    cudaFree(r.a); cudaFree(r.fwi); cudaFree(r.sfi); cudaFree(r.id); cudaFree(r.sco);
    r.a = a; r.b = a + 1; r.fwi = fwi; r.sfi = sfi; r.id = id; r.sco = sco; r.cap = cap;
    return ALB_OK;
}

static void release_records(AlbCtx* ctx, int c) {
    RecordStore& r = ctx->rec[c];
    cudaFree(r.a); cudaFree(r.fwi); cudaFree(r.sfi); cudaFree(r.id); cudaFree(r.sco);
    r = RecordStore{};
}

// Bring a channel's records back into an append store (from its index) before appending.
static int restore_records(AlbCtx* ctx, int c, uint64_t need) {
    if (!ctx->rec_released[c]) return ALB_OK;
    const uint64_t n = ctx->h_rec_count[c];
    int rc = ensure_records(ctx, c, need, 0);
    if (rc) return rc;
    const MapIndex& m = ctx->map[c];
    RecordStore& r = ctx->rec[c];
    if (n) {
        // the index holds the halves in two arrays; the store interleaves them (32-byte pitch)
        CK(cudaMemcpy2DAsync(r.a, 32, m.a, 16, 16, n, cudaMemcpyDeviceToDevice, ctx->st));
        CK(cudaMemcpy2DAsync(r.b, 32, m.b, 16, 16, n, cudaMemcpyDeviceToDevice, ctx->st));
        if (r.fwi && m.fwi) {
            CK(cudaMemcpyAsync(r.fwi, m.fwi, n * 16, cudaMemcpyDeviceToDevice, ctx->st));
            CK(cudaMemcpyAsync(r.sfi, m.sfi, n * 16, cudaMemcpyDeviceToDevice, ctx->st));
        }
        if (r.id && m.id) CK(cudaMemcpyAsync(r.id, m.id, n * 4, cudaMemcpyDeviceToDevice, ctx->st));
        if (r.sco && m.sco) CK(cudaMemcpyAsync(r.sco, m.sco, n * 16, cudaMemcpyDeviceToDevice, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    ctx->rec_released[c] = false;
    return ALB_OK;
}

static int ensure_queries(AlbCtx* ctx, int k, uint64_t need) {
    if (ctx->qcap[k] >= need && (!ctx->keep_ids || ctx->qid[k]) && (!ctx->sc.adjoint || ctx->qs[k])) return ALB_OK;
    uint64_t cap = std::max<uint64_t>(need + need / 4, 1024);
    CK(cudaStreamSynchronize(ctx->st));
    cudaFree(ctx->qa[k]); cudaFree(ctx->qb[k]); cudaFree(ctx->qc[k]); cudaFree(ctx->qid[k]); cudaFree(ctx->qperm[k]);
    cudaFree(ctx->qrk[k][0]); cudaFree(ctx->qrk[k][1]); cudaFree(ctx->qs[k]);
    ctx->qa[k] = ctx->qb[k] = ctx->qc[k] = nullptr; ctx->qperm[k] = nullptr;
    ctx->qid[k] = nullptr; ctx->qrk[k][0] = ctx->qrk[k][1] = nullptr; ctx->qs[k] = nullptr;
    ctx->qcap[k] = 0;
    CK(cudaMalloc(&ctx->qa[k], cap * 16));
    CK(cudaMalloc(&ctx->qb[k], cap * 16));
    CK(cudaMalloc(&ctx->qc[k], cap * 16));
    CK(cudaMalloc(&ctx->qperm[k], cap * 4));
    if (ctx->keep_ids) {
        CK(cudaMalloc(&ctx->qid[k], cap * 4));
        CK(cudaMalloc(&ctx->qrk[k][0], cap * 8));
        CK(cudaMalloc(&ctx->qrk[k][1], cap * 8));
    }
    if (ctx->sc.adjoint) CK(cudaMalloc(&ctx->qs[k], cap * 16));
    ctx->qcap[k] = cap;
    return ALB_OK;
}

static TraceOut make_out(AlbCtx* ctx) {
    TraceOut o{};
    for (int c = 0; c < ALB_CHANNELS; ++c) {
        o.rec_a[c] = ctx->rec[c].a;
        o.rec_b[c] = ctx->rec[c].b;
        o.rec_fwi[c] = ctx->rec[c].fwi;
        o.rec_sfi[c] = ctx->rec[c].sfi;
        o.rec_id[c] = ctx->rec[c].id;
        o.rec_sco[c] = ctx->sc.adjoint ? ctx->rec[c].sco : nullptr;
        o.rec_cap[c] = ctx->rec[c].cap;
    }
    o.rec_count = ctx->d_rec_count;
    for (int k = 0; k < 3; ++k) {
        o.q_a[k] = ctx->qa[k];
        o.q_b[k] = ctx->qb[k];
        o.q_c[k] = ctx->qc[k];
        o.q_id[k] = ctx->qid[k];
        o.q_s[k] = ctx->sc.adjoint ? ctx->qs[k] : nullptr;
        o.q_cap[k] = ctx->qcap[k];
    }
    o.q_count = ctx->d_q_count;
    o.ex_pos = ctx->keep_exit ? ctx->ex_pos : nullptr;
    o.ex_dir = ctx->ex_dir;
    o.ex_f = ctx->ex_f;
    o.hm_radius = ctx->hm_radius;
    o.err = ctx->d_err;
    o.stats = ctx->d_stats;
    return o;
}

// Q9 of the reference: a gather on a map with fewer than k records raises IndexError.
static int check_map_sizes(AlbCtx* ctx) {
    static const int need[3][2] = {{ALB_BOTTOM_REFLECTION, -1}, {ALB_SCATTER, -1},
                                   {ALB_SURFACE_REFLECTION, ALB_SURFACE_TRANSMISSION_UP}};
    static const char* names[4] = {"BOTTOM_REFLECTION", "SCATTER", "SURFACE_REFLECTION", "SURFACE_TRANSMISSION_UP"};
    for (int k = 0; k < 3; ++k) {
        if (ctx->h_q_count[k] == 0) continue;
        for (int j = 0; j < 2; ++j) {
            int c = need[k][j];
            if (c < 0) continue;
            if (ctx->map[c].n_real < (uint64_t)ctx->sc.k) {
                char buf[256];
                snprintf(buf, sizeof buf, "photon map %s holds %llu records, fewer than k=%d", names[c],
                         (unsigned long long)ctx->map[c].n_real, ctx->sc.k);
                return fail(ctx, ALB_ERR_TOO_FEW, buf);
            }
        }
    }
    return ALB_OK;
}

extern "C" int alb_trace(AlbCtx* ctx, int pass, uint64_t n, uint64_t seed, uint64_t first, const AlbReplay* rp) {
    if (!ctx) return ALB_ERR_INVALID;
    if (pass != ALB_FORWARD && pass != ALB_BACKWARD) return fail(ctx, ALB_ERR_INVALID, "pass must be 0 or 1");
    if (pass == ALB_BACKWARD && !ctx->maps_built) return fail(ctx, ALB_ERR_STATE, "backward trace before alb_build_maps");
    if (first + n > (1ull << 32)) return fail(ctx, ALB_ERR_INVALID, "photon ids are 32-bit per pass");
    if (rp && ctx->sc.slope_sigma > 0.0)
        return fail(ctx, ALB_ERR_INVALID, "surface slopes draw variates the reference never records (Philox only)");
    CK(cudaSetDevice(ctx->device));
    ctx->err.clear();
    // replay streams to the device
    AlbReplay drp{};
    size_t mark = ctx->ws.mark();
    if (rp) {
        if (!rp->offsets || !rp->values || !rp->tau) return fail(ctx, ALB_ERR_INVALID, "incomplete replay");
        int64_t* o = (int64_t*)ctx->ws.take_bytes((n + 1) * 8);
        double* v = (double*)ctx->ws.take_bytes(rp->n_values * 8 + 8);
        float* t = (float*)ctx->ws.take_bytes(rp->n_values * 4 + 4);
        if (!o || !v || !t) return fail(ctx, ALB_ERR_CUDA, "replay upload allocation failed");
        CK(cudaMemcpyAsync(o, rp->offsets, (n + 1) * 8, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaMemcpyAsync(v, rp->values, rp->n_values * 8, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaMemcpyAsync(t, rp->tau, rp->n_values * 4, cudaMemcpyHostToDevice, ctx->st));
        drp.offsets = o;
        drp.values = v;
        drp.tau = t;
        drp.n_values = rp->n_values;
    }
    if (ctx->keep_exit) {
        if (ctx->ex_cap < n) {
            cudaFree(ctx->ex_pos); cudaFree(ctx->ex_dir); cudaFree(ctx->ex_f);
            CK(cudaMalloc(&ctx->ex_pos, n * 24));
            CK(cudaMalloc(&ctx->ex_dir, n * 24));
            CK(cudaMalloc(&ctx->ex_f, n * 40));
            ctx->ex_cap = n;
        }
        ctx->ex_n = n;
    }
    // slots 28/29 keep the last forward trace's events and photons across the backward trace
    CK(cudaMemsetAsync(ctx->d_stats, 0, 28 * 8, ctx->st));
    CK(cudaMemsetAsync(ctx->d_stats + 30, 0, 8, ctx->st));
    if (pass == ALB_FORWARD) {
        ctx->maps_built = false;
        uint64_t before[ALB_CHANNELS];
        std::memcpy(before, ctx->h_rec_count, sizeof before);
        std::vector<unsigned> radius_backup;
        size_t hb = ctx->sc.heatmap ? (size_t)ctx->sc.hm_bins * ctx->sc.hm_bins : 0;
        for (int attempt = 0; attempt < 3; ++attempt) {
            for (int c = 0; c < ALB_CHANNELS; ++c) {
                uint64_t est = (uint64_t)(ctx->rec_rate[c] * (double)n * 1.03) + 4096;
                if (ctx->map_cap_hint > 0) est = std::max<uint64_t>(est, (uint64_t)ctx->map_cap_hint);
                int rc = ctx->rec_released[c] ? restore_records(ctx, c, before[c] + est)
                                               : ensure_records(ctx, c, before[c] + est, before[c]);
                if (rc) return rc;
            }
            if (hb && attempt == 0) {
                radius_backup.resize(hb);
                CK(cudaMemcpyAsync(radius_backup.data(), ctx->hm_radius, hb * 4, cudaMemcpyDeviceToHost, ctx->st));
            }
            TraceOut o = make_out(ctx);
            PhaseTimer pt(ctx, 0);
            launch_trace(ctx->sc, o, ALB_FORWARD, n, first, seed, rp ? &drp : nullptr, &ctx->launches, ctx->st,
                         ctx->precise ? nullptr : &ctx->fast);
            pt.stop();
            int rc = check_device(ctx, "forward trace");
            if (rc) return rc;
            unsigned long long cnt[ALB_CHANNELS];
            CK(cudaMemcpyAsync(cnt, ctx->d_rec_count, sizeof cnt, cudaMemcpyDeviceToHost, ctx->st));
            CK(cudaStreamSynchronize(ctx->st));
            bool overflow = false;
            for (int c = 0; c < ALB_CHANNELS; ++c) {
                uint64_t added = cnt[c] - before[c];
                if (n > 0) ctx->rec_rate[c] = std::max(ctx->rec_rate[c] * 0.5, (double)added / (double)n);
                if (cnt[c] > ctx->rec[c].cap) overflow = true;
            }
            if (!overflow) {
                for (int c = 0; c < ALB_CHANNELS; ++c) ctx->h_rec_count[c] = cnt[c];
                CK(cudaMemcpyAsync(ctx->d_stats + 28, ctx->d_stats, 2 * 8, cudaMemcpyDeviceToDevice, ctx->st));
                ctx->ws.release(mark);
                return ALB_OK;
            }
            // undo and retry with the measured sizes
            CK(cudaMemsetAsync(ctx->d_stats, 0, 2 * 8, ctx->st));
            CK(cudaMemcpyAsync(ctx->d_rec_count, before, sizeof before, cudaMemcpyHostToDevice, ctx->st));
            if (hb) CK(cudaMemcpyAsync(ctx->hm_radius, radius_backup.data(), hb * 4, cudaMemcpyHostToDevice, ctx->st));
            CK(cudaStreamSynchronize(ctx->st));
            for (int c = 0; c < ALB_CHANNELS; ++c) ctx->rec_rate[c] = (double)(cnt[c] - before[c]) / (double)n;
        }
        return fail(ctx, ALB_ERR_CAPACITY, "photon-map capacity could not be established");
    }
    // backward: trace -> queries -> gathers. Without per-photon exports the photons go in
    // chunks, so that query buffers stay bounded whatever n is (the waveform sums are
    // integer and order independent, so chunking cannot change the result).
    Accum acc{};
    acc.wf_lo = ctx->wf;
    acc.wf_hi = ctx->wf + (size_t)ALB_CHANNELS * ctx->sc.nbins;
    acc.nbins = ctx->sc.nbins;
    if (ctx->sc.adjoint) {
        acc.jac_lo = ctx->jac;
        acc.jac_hi = ctx->jac + (size_t)kJacParams * ALB_CHANNELS * ctx->sc.nbins;
    }
    if (ctx->sc.heatmap) {
        size_t hb = (size_t)ctx->sc.hm_bins * ctx->sc.hm_bins;
        acc.hw_lo = ctx->hm;
        acc.hw_hi = ctx->hm + hb;
        acc.hf_lo = ctx->hm + 2 * hb;
        acc.hf_hi = ctx->hm + 3 * hb;
    }
    const bool chunked = !ctx->keep_exit && !ctx->keep_ids && !rp;
    const uint64_t chunk = chunked ? kBackwardChunk : std::max<uint64_t>(n, 1);
    for (uint64_t c0 = 0; c0 == 0 || c0 < n; c0 += chunk) {
        const uint64_t nc = std::min<uint64_t>(chunk, n - c0);
        for (int attempt = 0; attempt < 3; ++attempt) {
            for (int k = 0; k < 3; ++k) {
                uint64_t est = (uint64_t)(ctx->q_rate[k] * (double)nc * 1.1) + 4096;
                int rc = ensure_queries(ctx, k, est);
                if (rc) return rc;
            }
            CK(cudaMemsetAsync(ctx->d_q_count, 0, 3 * 8, ctx->st));
            TraceOut o = make_out(ctx);
            PhaseTimer pt(ctx, 2);
            launch_trace(ctx->sc, o, ALB_BACKWARD, nc, first + c0, seed, rp ? &drp : nullptr, &ctx->launches,
                         ctx->st, ctx->precise ? nullptr : &ctx->fast);
            pt.stop();
            int rc = check_device(ctx, "backward trace");
            if (rc) return rc;
            unsigned long long cnt[3];
            CK(cudaMemcpyAsync(cnt, ctx->d_q_count, sizeof cnt, cudaMemcpyDeviceToHost, ctx->st));
            CK(cudaStreamSynchronize(ctx->st));
            bool overflow = false;
            for (int k = 0; k < 3; ++k) {
                if (nc > 0) ctx->q_rate[k] = std::max(ctx->q_rate[k] * 0.5, (double)cnt[k] / (double)nc);
                if (cnt[k] > ctx->qcap[k]) overflow = true;
                ctx->h_q_count[k] = cnt[k];
            }
            if (!overflow) break;
            for (int k = 0; k < 3; ++k) ctx->q_rate[k] = (double)cnt[k] / (double)nc;
            if (attempt == 2) return fail(ctx, ALB_ERR_CAPACITY, "query capacity could not be established");
        }
        int rc = ctx->sc.radius > 0.0 ? ALB_OK : check_map_sizes(ctx);  // k-NN needs k records
        if (rc) return rc;
        static const int kinds[4] = {kQueryBottom, kQueryScatter, kQuerySurface, kQuerySurface};
        static const int chans[4] = {ALB_BOTTOM_REFLECTION, ALB_SCATTER, ALB_SURFACE_REFLECTION,
                                     ALB_SURFACE_TRANSMISSION_UP};
        for (int g = 0; g < 4; ++g) {
            int k = kinds[g], c = chans[g];
            uint64_t nq = ctx->h_q_count[k];
            if (nq == 0) continue;
            QueryDev q{};
            q.a = ctx->qa[k];
            q.b = ctx->qb[k];
            q.c = ctx->qc[k];
            q.s = ctx->sc.adjoint ? ctx->qs[k] : nullptr;
            q.n = nq;
            q.rk_out = ctx->keep_ids ? ctx->qrk[k][g == 3 ? 1 : 0] : nullptr;
            q.stats = ctx->d_stats + 4 + 4 * c;  // per channel: leaves, nodes, selects, queries
            q.inexact = ctx->d_stats + 24 + c;
            q.retries = ctx->d_stats + 30;
            if (ctx->sort_q) {
                PhaseTimer ps(ctx, 3);
                const int src = sort_queries(ctx->ws, ctx->qa[k], nq, ctx->qperm[k], ctx->st);
                ps.stop();
                if (src != 0) return fail(ctx, ALB_ERR_CUDA, "query sort: device memory allocation failed");
                q.perm = ctx->qperm[k];
            }
            PhaseTimer pg(ctx, 4 + c);
            launch_gather(ctx->sc, map_dev(ctx->map[c]), q, c, acc, ctx->d_err, &ctx->launches, ctx->st);
            pg.stop();
            ctx->gathered[c] += (int64_t)nq;
        }
        rc = check_device(ctx, "gather");
        if (rc) return rc;
        if (n == 0) break;
    }
    ctx->ws.release(mark);
    return ALB_OK;
}

extern "C" int alb_build_maps(AlbCtx* ctx) {
    if (!ctx) return ALB_ERR_INVALID;
    CK(cudaSetDevice(ctx->device));
    PhaseTimer pt(ctx, 1);
    for (int c = 0; c < ALB_CHANNELS; ++c) {
        if (ctx->rec_released[c]) continue;  // already indexed, nothing appended since
        RecordStore r = ctx->rec[c];
        if (!ctx->sc.adjoint) r.sco = nullptr;  // a store kept from an adjoint run: no scores now
        if (build_map_index(ctx->ws, r, ctx->h_rec_count[c], ctx->map[c], ctx->st) != 0)
            return fail(ctx, ALB_ERR_CAPACITY, "photon-map index build failed (device memory or partition)");
        CK(cudaStreamSynchronize(ctx->st));
        if (ctx->keep_records) continue;  // the store stays for the next simulation
        release_records(ctx, c);
        ctx->rec_released[c] = true;
    }
    pt.stop();
    int rc = check_device(ctx, "map build");
    if (rc) return rc;
    ctx->maps_built = true;
    return ALB_OK;
}

extern "C" int alb_map_size(AlbCtx* ctx, int c, uint64_t* out) {
    if (!ctx || !out || c < 0 || c >= ALB_CHANNELS) return ALB_ERR_INVALID;
    *out = ctx->h_rec_count[c];
    return ALB_OK;
}

extern "C" int alb_export_map(AlbCtx* ctx, int c, float* pos, float* dir, float* energy, float* time,
                              float* fwi, float* sfi, int64_t* pid, size_t n) {
    if (!ctx || c < 0 || c >= ALB_CHANNELS) return ALB_ERR_INVALID;
    uint64_t m = ctx->h_rec_count[c];
    if (n < m) return fail(ctx, ALB_ERR_INVALID, "export buffer smaller than the map");
    if (m == 0) return ALB_OK;
    const float4 *a, *b, *fw, *sf;
    const uint32_t* id;
    size_t pitch;  // bytes between consecutive records' a (and b) halves
    // records in append order (the interleaved store), or in index order once the channel
    // has been indexed
    if (ctx->rec_released[c]) {
        const MapIndex& mi = ctx->map[c];
        a = mi.a; b = mi.b; id = mi.id; fw = mi.fwi; sf = mi.sfi;
        pitch = 16;
    } else {
        a = ctx->rec[c].a; b = ctx->rec[c].b; id = ctx->rec[c].id; fw = ctx->rec[c].fwi; sf = ctx->rec[c].sfi;
        pitch = 32;
    }
    std::vector<float4> ha(m), hb(m), hf, hs;
    CK(cudaMemcpy2D(ha.data(), 16, a, pitch, 16, m, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy2D(hb.data(), 16, b, pitch, 16, m, cudaMemcpyDeviceToHost));
    if (fw && (fwi || sfi)) {
        hf.resize(m);
        hs.resize(m);
        CK(cudaMemcpy(hf.data(), fw, m * 16, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hs.data(), sf, m * 16, cudaMemcpyDeviceToHost));
    }
    std::vector<uint32_t> hid;
    if (pid && id) {
        hid.resize(m);
        CK(cudaMemcpy(hid.data(), id, m * 4, cudaMemcpyDeviceToHost));
    }
    const float qnan = std::nanf("");
    for (uint64_t i = 0; i < m; ++i) {
        if (pos) { pos[3 * i] = ha[i].x; pos[3 * i + 1] = ha[i].y; pos[3 * i + 2] = ha[i].z; }
        if (energy) energy[i] = ha[i].w;
        if (dir) { dir[3 * i] = hb[i].x; dir[3 * i + 1] = hb[i].y; dir[3 * i + 2] = hb[i].z; }
        if (time) time[i] = hb[i].w;
        if (fwi) {
            fwi[3 * i] = hf.empty() ? qnan : hf[i].x;
            fwi[3 * i + 1] = hf.empty() ? qnan : hf[i].y;
            fwi[3 * i + 2] = hf.empty() ? qnan : hf[i].z;
        }
        if (sfi) {
            sfi[3 * i] = hs.empty() ? qnan : hs[i].x;
            sfi[3 * i + 1] = hs.empty() ? qnan : hs[i].y;
            sfi[3 * i + 2] = hs.empty() ? qnan : hs[i].z;
        }
        if (pid) pid[i] = hid.empty() ? -1 : (int64_t)hid[i];
    }
    return ALB_OK;
}

extern "C" int alb_get_heatmaps(AlbCtx* ctx, double* water, double* seafloor, float* radius, size_t bins2) {
    if (!ctx) return ALB_ERR_INVALID;
    if (!ctx->sc.heatmap) return fail(ctx, ALB_ERR_STATE, "heatmaps are disabled in this scene");
    size_t hb = (size_t)ctx->sc.hm_bins * ctx->sc.hm_bins;
    if (bins2 < hb) return fail(ctx, ALB_ERR_INVALID, "heatmap buffer too small");
    std::vector<unsigned long long> h(4 * hb);
    CK(cudaMemcpy(h.data(), ctx->hm, 4 * hb * 8, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < hb; ++i) {
        if (water) water[i] = fix_to_double(h[i], (long long)h[hb + i]);
        if (seafloor) seafloor[i] = fix_to_double(h[2 * hb + i], (long long)h[3 * hb + i]);
    }
    if (radius) {
        std::vector<unsigned> r(hb);
        CK(cudaMemcpy(r.data(), ctx->hm_radius, hb * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < hb; ++i) radius[i] = (float)r[i];
    }
    return ALB_OK;
}

static int read_wf(AlbCtx* ctx, int c, std::vector<double>& out) {
    int64_t nb = ctx->sc.nbins;
    std::vector<unsigned long long> lo(nb), hi(nb);
    CK(cudaMemcpyAsync(lo.data(), ctx->wf + (size_t)c * nb, nb * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hi.data(), ctx->wf + (size_t)ALB_CHANNELS * nb + (size_t)c * nb, nb * 8, cudaMemcpyDeviceToHost,
                       ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    out.resize(nb);
    for (int64_t i = 0; i < nb; ++i) out[i] = fix_to_double(lo[i], (long long)hi[i]);
    return ALB_OK;
}

extern "C" int alb_get_waveform(AlbCtx* ctx, int c, float* out, size_t nbins) {
    if (!ctx || !out || c < 0 || c >= ALB_CHANNELS) return ALB_ERR_INVALID;
    if (nbins < (size_t)ctx->sc.nbins) return fail(ctx, ALB_ERR_INVALID, "waveform buffer too small");
    std::vector<double> w;
    int rc = read_wf(ctx, c, w);
    if (rc) return rc;
    for (size_t i = 0; i < w.size(); ++i) out[i] = (float)w[i];
    return ALB_OK;
}

extern "C" int alb_get_waveform_f64(AlbCtx* ctx, int c, double* out, size_t nbins) {
    if (!ctx || !out || c < 0 || c >= ALB_CHANNELS) return ALB_ERR_INVALID;
    if (nbins < (size_t)ctx->sc.nbins) return fail(ctx, ALB_ERR_INVALID, "waveform buffer too small");
    std::vector<double> w;
    int rc = read_wf(ctx, c, w);
    if (rc) return rc;
    std::memcpy(out, w.data(), w.size() * 8);
    return ALB_OK;
}

extern "C" int alb_get_jacobian(AlbCtx* ctx, int param, int c, double* out, size_t nbins) {
    if (!ctx || !out || c < 0 || c >= ALB_CHANNELS) return ALB_ERR_INVALID;
    if (param == 0)
        return fail(ctx, ALB_ERR_INVALID, "the depth column is a host-side central difference (no score form)");
    if (param < 1 || param >= ALB_ADJ_PARAMS) return fail(ctx, ALB_ERR_INVALID, "unknown adjoint parameter");
    if (!ctx->jac) return fail(ctx, ALB_ERR_STATE, "ALB_OPT_ADJOINT is not enabled");
    const int64_t nb = ctx->sc.nbins;
    if (nbins < (size_t)nb) return fail(ctx, ALB_ERR_INVALID, "jacobian buffer too small");
    const size_t off = ((size_t)(param - 1) * ALB_CHANNELS + c) * nb;
    const size_t half = (size_t)kJacParams * ALB_CHANNELS * nb;
    std::vector<unsigned long long> lo(nb), hi(nb);
    CK(cudaMemcpyAsync(lo.data(), ctx->jac + off, nb * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hi.data(), ctx->jac + half + off, nb * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int64_t i = 0; i < nb; ++i) out[i] = fix_to_double(lo[i], (long long)hi[i]);
    return ALB_OK;
}

extern "C" int alb_adjoint(AlbCtx* ctx, const double* dL_dw, size_t nbins, double* grad) {
    if (!ctx || !dL_dw || !grad) return ALB_ERR_INVALID;
    const int64_t nb = ctx->sc.nbins;
    if (nbins != (size_t)nb) return fail(ctx, ALB_ERR_INVALID, "dL_dw must hold channels * nbins values");
    grad[0] = std::nan("");
    std::vector<double> j(nb);
    for (int p = 1; p < ALB_ADJ_PARAMS; ++p) {
        double acc = 0.0;
        for (int c = 0; c < ALB_CHANNELS; ++c) {
            int rc = alb_get_jacobian(ctx, p, c, j.data(), nb);
            if (rc) return rc;
            for (int64_t i = 0; i < nb; ++i) acc += dL_dw[(size_t)c * nb + i] * j[i];
        }
        grad[p] = acc;
    }
    return ALB_OK;
}

extern "C" int alb_export_map_scores(AlbCtx* ctx, int c, float* scores, size_t n) {
    if (!ctx || !scores || c < 0 || c >= ALB_CHANNELS) return ALB_ERR_INVALID;
    if (!ctx->sc.adjoint) return fail(ctx, ALB_ERR_STATE, "ALB_OPT_ADJOINT is not enabled");
    const uint64_t m = ctx->h_rec_count[c];
    if (n < m) return fail(ctx, ALB_ERR_INVALID, "export buffer smaller than the map");
    if (m == 0) return ALB_OK;
    const float4* s = ctx->rec_released[c] ? ctx->map[c].sco : ctx->rec[c].sco;
    if (!s) return fail(ctx, ALB_ERR_STATE, "records carry no scores");
    CK(cudaMemcpy(scores, s, m * 16, cudaMemcpyDeviceToHost));
    return ALB_OK;
}

extern "C" int alb_reset_waveform(AlbCtx* ctx) {
    if (!ctx) return ALB_ERR_INVALID;
    CK(cudaMemsetAsync(ctx->wf, 0, (size_t)2 * ALB_CHANNELS * ctx->sc.nbins * 8, ctx->st));
    if (ctx->hm) CK(cudaMemsetAsync(ctx->hm, 0, (size_t)4 * ctx->sc.hm_bins * ctx->sc.hm_bins * 8, ctx->st));
    if (ctx->jac)
        CK(cudaMemsetAsync(ctx->jac, 0, (size_t)2 * kJacParams * ALB_CHANNELS * ctx->sc.nbins * 8, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return ALB_OK;
}

extern "C" int alb_reset(AlbCtx* ctx) {
    if (!ctx) return ALB_ERR_INVALID;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemsetAsync(ctx->d_rec_count, 0, ALB_CHANNELS * 8, ctx->st));
    CK(cudaMemsetAsync(ctx->d_q_count, 0, 3 * 8, ctx->st));
    if (ctx->hm_radius)
        CK(cudaMemsetAsync(ctx->hm_radius, 0, (size_t)ctx->sc.hm_bins * ctx->sc.hm_bins * 4, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int c = 0; c < ALB_CHANNELS; ++c) {
        ctx->h_rec_count[c] = 0;
        release_map_index(ctx->map[c]);  // an empty simulation holds no index memory
        ctx->map[c].n = 0;
        ctx->map[c].n_real = 0;
        ctx->rec_released[c] = false;
    }
    for (int k = 0; k < 3; ++k) ctx->h_q_count[k] = 0;
    ctx->maps_built = false;
    ctx->ex_n = 0;
    return alb_reset_waveform(ctx);
}

extern "C" int alb_export_exit_states(AlbCtx* ctx, double* pos, double* dir, float* energy, float* tau,
                                      float* tau_target, float* time, float* fwi, float* sfi, size_t n) {
    if (!ctx) return ALB_ERR_INVALID;
    if (!ctx->keep_exit || ctx->ex_n == 0) return fail(ctx, ALB_ERR_STATE, "no exit states kept");
    if (n < ctx->ex_n) return fail(ctx, ALB_ERR_INVALID, "exit-state buffer too small");
    uint64_t m = ctx->ex_n;
    std::vector<float> f(10 * m);
    if (pos) CK(cudaMemcpy(pos, ctx->ex_pos, m * 24, cudaMemcpyDeviceToHost));
    if (dir) CK(cudaMemcpy(dir, ctx->ex_dir, m * 24, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(f.data(), ctx->ex_f, m * 40, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < m; ++i) {
        const float* r = f.data() + 10 * i;
        if (energy) energy[i] = r[0];
        if (tau) tau[i] = r[1];
        if (tau_target) tau_target[i] = r[2];
        if (time) time[i] = r[3];
        for (int j = 0; j < 3; ++j) {
            if (fwi) fwi[3 * i + j] = r[4 + j];
            if (sfi) sfi[3 * i + j] = r[7 + j];
        }
    }
    return ALB_OK;
}

extern "C" int alb_query_count(AlbCtx* ctx, int kind, uint64_t* out) {
    if (!ctx || !out || kind < 0 || kind > 2) return ALB_ERR_INVALID;
    *out = ctx->h_q_count[kind];
    return ALB_OK;
}

extern "C" int alb_export_queries(AlbCtx* ctx, int kind, double* pos, float* dir, float* energy, float* time,
                                  int64_t* pid, double* rk, double* rk2, size_t n) {
    if (!ctx || kind < 0 || kind > 2) return ALB_ERR_INVALID;
    uint64_t m = ctx->h_q_count[kind];
    if (n < m) return fail(ctx, ALB_ERR_INVALID, "query buffer too small");
    if (m == 0) return ALB_OK;
    std::vector<float4> a(m), b(m), c(m);
    CK(cudaMemcpy(a.data(), ctx->qa[kind], m * 16, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(b.data(), ctx->qb[kind], m * 16, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(c.data(), ctx->qc[kind], m * 16, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> id;
    if (ctx->qid[kind]) {
        id.resize(m);
        CK(cudaMemcpy(id.data(), ctx->qid[kind], m * 4, cudaMemcpyDeviceToHost));
    }
    if (rk && ctx->qrk[kind][0]) CK(cudaMemcpy(rk, ctx->qrk[kind][0], m * 8, cudaMemcpyDeviceToHost));
    if (rk2 && ctx->qrk[kind][1]) CK(cudaMemcpy(rk2, ctx->qrk[kind][1], m * 8, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < m; ++i) {
        if (pos) {
            pos[3 * i] = (double)a[i].x + (double)c[i].x;
            pos[3 * i + 1] = (double)a[i].y + (double)c[i].y;
            pos[3 * i + 2] = (double)a[i].z + (double)c[i].z;
        }
        if (dir) { dir[3 * i] = b[i].x; dir[3 * i + 1] = b[i].y; dir[3 * i + 2] = b[i].z; }
        if (energy) energy[i] = a[i].w;
        if (time) time[i] = b[i].w;
        if (pid) pid[i] = id.empty() ? -1 : (int64_t)id[i];
    }
    return ALB_OK;
}

extern "C" int alb_knn(AlbCtx* ctx, const float* pts, uint64_t m, const double* qs, uint64_t nq, int k,
                       int32_t* idx, double* dist) {
    if (!ctx || !pts || !qs || !idx || !dist || k < 1 || k > 256) return ALB_ERR_INVALID;
    if (m < (uint64_t)k) return fail(ctx, ALB_ERR_TOO_FEW, "fewer points than k");
    CK(cudaSetDevice(ctx->device));
    // the record's w lane carries its original index (bit pattern) through the sort
    std::vector<float4> ha(m);
    for (uint64_t i = 0; i < m; ++i) {
        uint32_t tag = (uint32_t)i;
        float w;
        std::memcpy(&w, &tag, 4);
        ha[i] = make_float4(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], w);
    }
    RecordStore r{};
    size_t mark = ctx->ws.mark();
    r.a = (float4*)ctx->ws.take_bytes(m * 32);  // interleaved store (RecordStore)
    r.b = r.a ? r.a + 1 : nullptr;
    double* dq = (double*)ctx->ws.take_bytes(nq * 24);
    int32_t* di = (int32_t*)ctx->ws.take_bytes(nq * k * 4);
    double* dd = (double*)ctx->ws.take_bytes(nq * k * 8);
    if (!r.a || !dq || !di || !dd) return fail(ctx, ALB_ERR_CUDA, "knn allocation failed");
    CK(cudaMemsetAsync(r.a, 0, m * 32, ctx->st));
    CK(cudaMemcpy2DAsync(r.a, 32, ha.data(), 16, 16, m, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(dq, qs, nq * 24, cudaMemcpyHostToDevice, ctx->st));
    MapIndex mi;
    if (build_map_index(ctx->ws, r, m, mi, ctx->st) != 0) return fail(ctx, ALB_ERR_CAPACITY, "knn index build failed");
    // indices returned by the search refer to the sorted order: map them back
    launch_knn(map_dev(mi), dq, nq, k, di, dd, ctx->d_err, ctx->st);
    std::vector<int32_t> sorted_idx(nq * k);
    int rc = check_device(ctx, "knn");
    if (rc) {
        cudaFree(mi.a); cudaFree(mi.b); cudaFree(mi.box_lo); cudaFree(mi.box_hi);
        ctx->ws.release(mark);
        return rc;
    }
    CK(cudaMemcpy(sorted_idx.data(), di, nq * k * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dist, dd, nq * k * 8, cudaMemcpyDeviceToHost));
    std::vector<float4> sa(mi.n);  // the index may hold more slots than points
    CK(cudaMemcpy(sa.data(), mi.a, mi.n * 16, cudaMemcpyDeviceToHost));
    cudaFree(mi.a); cudaFree(mi.b); cudaFree(mi.box_lo); cudaFree(mi.box_hi);
    ctx->ws.release(mark);
    for (uint64_t i = 0; i < nq * (uint64_t)k; ++i) {
        uint32_t tag;
        std::memcpy(&tag, &sa[sorted_idx[i]].w, 4);
        idx[i] = (int32_t)tag;
    }
    return ALB_OK;
}

extern "C" int alb_stats(AlbCtx* ctx, int64_t* out, int n) {
    if (!ctx || !out) return ALB_ERR_INVALID;
    unsigned long long s[32];
    CK(cudaMemcpy(s, ctx->d_stats, sizeof s, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n && i < 32; ++i) out[i] = (int64_t)s[i];
    if (n > 2) out[2] = launches_total();
    return ALB_OK;
}

extern "C" int alb_phase_times(AlbCtx* ctx, double* ms, int64_t* calls, int64_t* gathers, int reset) {
    if (!ctx) return ALB_ERR_INVALID;
    for (int i = 0; i < ALB_PHASES; ++i) {
        if (ms) ms[i] = ctx->phase_ms[i];
        if (calls) calls[i] = ctx->phase_calls[i];
    }
    if (gathers)
        for (int c = 0; c < ALB_CHANNELS; ++c) gathers[c] = ctx->gathered[c];
    if (reset) {
        for (int i = 0; i < ALB_PHASES; ++i) {
            ctx->phase_ms[i] = 0.0;
            ctx->phase_calls[i] = 0;
        }
        for (int c = 0; c < ALB_CHANNELS; ++c) ctx->gathered[c] = 0;
    }
    return ALB_OK;
}

// ------------------------------------------------------------------------------------------
// Batched instances (extension)
// ------------------------------------------------------------------------------------------

// Empty the context for the next instance without releasing device memory: stream-ordered
// memsets only, so the other workers' streams keep running.
static int soft_reset(AlbCtx* ctx) {
    const size_t nb = (size_t)ctx->sc.nbins;
    CK(cudaMemsetAsync(ctx->d_rec_count, 0, ALB_CHANNELS * 8, ctx->st));
    CK(cudaMemsetAsync(ctx->d_q_count, 0, 3 * 8, ctx->st));
    CK(cudaMemsetAsync(ctx->wf, 0, 2 * ALB_CHANNELS * nb * 8, ctx->st));
    if (ctx->jac) CK(cudaMemsetAsync(ctx->jac, 0, (size_t)2 * kJacParams * ALB_CHANNELS * nb * 8, ctx->st));
    if (ctx->sc.heatmap) {
        const size_t hb = (size_t)ctx->sc.hm_bins * ctx->sc.hm_bins;
        CK(cudaMemsetAsync(ctx->hm, 0, 4 * hb * 8, ctx->st));
        CK(cudaMemsetAsync(ctx->hm_radius, 0, hb * 4, ctx->st));
    }
    CK(cudaStreamSynchronize(ctx->st));
    for (int c = 0; c < ALB_CHANNELS; ++c) {
        ctx->h_rec_count[c] = 0;
        ctx->map[c].n = 0;
        ctx->map[c].n_real = 0;
        ctx->map[c].nlevels = 0;
    }
    for (int k = 0; k < 3; ++k) ctx->h_q_count[k] = 0;
    ctx->maps_built = false;
    ctx->ex_n = 0;
    return ALB_OK;
}

static int run_instance(AlbCtx* ctx, AlbBatchInstance& I, int adjoint) {
    int rc = alb_trace(ctx, ALB_FORWARD, I.n_forward, I.seed, 0, nullptr);
    if (!rc) rc = alb_build_maps(ctx);
    if (!rc) rc = alb_trace(ctx, ALB_BACKWARD, I.n_backward, I.seed, 0, nullptr);
    if (rc) return rc;
    const int64_t nb = ctx->sc.nbins;
    std::vector<double> w;
    for (int c = 0; c < ALB_CHANNELS && !rc; ++c) {
        rc = read_wf(ctx, c, w);
        if (!rc && I.waveform) std::memcpy(I.waveform + (size_t)c * nb, w.data(), nb * 8);
    }
    if (!rc && adjoint && I.jacobian)
        for (int p = 1; p < ALB_ADJ_PARAMS && !rc; ++p)
            for (int c = 0; c < ALB_CHANNELS && !rc; ++c)
                rc = alb_get_jacobian(ctx, p, c, I.jacobian + ((size_t)(p - 1) * ALB_CHANNELS + c) * nb, nb);
    return rc;
}

extern "C" int alb_batch_run(AlbBatchInstance* inst, uint64_t n, const AlbBatchOptions* opt) {
    if (!inst || !opt) return ALB_ERR_INVALID;
    if (opt->streams < 1 || opt->streams > 64) {
        g_create_error = "streams must be in [1, 64]";
        return ALB_ERR_INVALID;
    }
    for (uint64_t i = 0; i < n; ++i)
        if (!inst[i].scene) {
            g_create_error = "instance without a scene";
            return ALB_ERR_INVALID;
        }
    // the work queue: largest instances first, so the uneven tail is short
    std::vector<uint64_t> order(n);
    for (uint64_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) {
        return inst[a].n_forward + inst[a].n_backward > inst[b].n_forward + inst[b].n_backward;
    });
    int64_t max_bins = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const AlbSceneParams* sp = inst[i].scene;
        max_bins = std::max<int64_t>(max_bins, sp->gate_bins > 0 ? sp->gate_bins : 2 * sp->steps);
    }
    std::atomic<uint64_t> next{0};
    std::mutex msg_mu;
    std::string last_msg;
    // Device-memory admission. A context keeps the buffers of the largest instance it ran,
    // so each worker holds an estimate of that footprint against a budget (80% of the free
    // memory at the start); a worker whose next instance needs more waits until the pool
    // has room or it is the only one running, and a worker dropping to instances a quarter
    // of its footprint releases its context. Footprint = forward photons x records per
    // photon (the largest seen so far x 1.5, 200 before any instance finished) x bytes per
    // record (append store, index, build temporaries; scores with the adjoint) + 64 MiB.
    cudaSetDevice(opt->device);
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const double budget = 0.8 * (double)free_b;
    const double bytes_per_record = opt->adjoint ? 162.0 : 130.0;
    std::mutex mem_mu;
    std::condition_variable mem_cv;
    double held_total = 0.0, rpp_seen = 0.0;
    int running = 0;
    int exclusive = 0;  // workers waiting to rerun an instance alone; the others hold no memory then
    auto need_of = [&](const AlbBatchInstance& I) {
        const double rpp = rpp_seen > 0.0 ? 1.5 * rpp_seen : 200.0;
        return (double)I.n_forward * rpp * bytes_per_record + 64.0 * 1048576.0;
    };
    auto worker = [&]() {
        cudaSetDevice(opt->device);
        double held = 0.0;
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) st = nullptr;
        AlbCtx* ctx = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        bool alone = false;  // the retry of an instance that ran out of memory beside others
        for (uint64_t t = next.fetch_add(1); t < n; t = alone ? t : next.fetch_add(1)) {
            AlbBatchInstance& I = inst[order[t]];
            I.device_ms = 0.f;
            int rc = ALB_OK;
            std::string msg;
            bool shared = false;  // other instances were running when this one started
            {
                std::unique_lock<std::mutex> g(mem_mu);
                const double need = need_of(I);
                auto drop_ctx = [&]() {  // release this worker's context and its device memory
                    g.unlock();
                    alb_destroy(ctx);
                    ctx = nullptr;
                    g.lock();
                    held_total -= held;
                    held = 0.0;
                    mem_cv.notify_all();
                };
                while (true) {
                    if (!alone && exclusive > 0) {  // another worker reruns an instance alone
                        if (ctx) drop_ctx();
                        mem_cv.wait(g, [&] { return exclusive == 0; });
                        continue;
                    }
                    if (ctx && held > (double)(1 << 30) && 4.0 * need < held) drop_ctx();  // small tail
                    const double grow = std::max(0.0, need - held);
                    mem_cv.wait(g, [&] {
                        if (!alone && exclusive > 0) return true;
                        // a rerun alone waits until no instance runs and every other worker
                        // has released its context (a worker that has just finished an
                        // instance still holds its buffers until it comes back here); this
                        // worker's own holding does not count
                        return alone ? (running == 0 && held_total - held <= 0.5)
                                     : (held_total + grow <= budget || running == 0);
                    });
                    if (!alone && exclusive > 0) continue;
                    held_total += grow;
                    held += grow;
                    shared = running > 0;
                    ++running;
                    break;
                }
            }
            if (!ctx) {
                rc = alb_create(I.scene, opt->device, &ctx);
                if (rc) {
                    msg = g_create_error;
                    ctx = nullptr;
                } else {
                    alb_set_option(ctx, ALB_OPT_STREAM, (int64_t)(intptr_t)st);
                    alb_set_option(ctx, ALB_OPT_PRECISE, opt->precise ? 1 : 0);
                    ctx->keep_records = true;
                    if (opt->adjoint) rc = alb_set_option(ctx, ALB_OPT_ADJOINT, 1);
                    if (!rc) {  // accumulators for the longest instance: no regrowth later
                        const int64_t own = ctx->sc.nbins;
                        ctx->sc.nbins = max_bins;
                        std::string e = ensure_accumulators(ctx);
                        ctx->sc.nbins = own;
                        if (!e.empty()) rc = fail(ctx, ALB_ERR_CUDA, e);
                        else if (cudaStreamSynchronize(ctx->st) != cudaSuccess) rc = fail(ctx, ALB_ERR_CUDA, "reserve");
                    }
                    if (rc) msg = ctx->err;
                }
            } else {
                std::string e = set_scene(ctx, I.scene);
                if (e.empty()) e = ensure_accumulators(ctx);
                if (!e.empty()) {
                    rc = ALB_ERR_INVALID;
                    msg = e;
                } else {
                    rc = soft_reset(ctx);
                    if (rc) msg = ctx->err;
                }
            }
            // with the adjoint option, an instance without a Jacobian buffer runs plain
            const int adj = opt->adjoint && I.jacobian ? 1 : 0;
            if (!rc && ctx && ctx->sc.adjoint != adj) {
                rc = alb_set_option(ctx, ALB_OPT_ADJOINT, adj);
                if (rc) msg = ctx->err;
            }
            if (!rc && ctx) {
                cudaEventRecord(e0, ctx->st);
                rc = run_instance(ctx, I, adj);
                cudaEventRecord(e1, ctx->st);
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&I.device_ms, e0, e1);
                if (rc) msg = ctx->err;
            }
            {
                std::lock_guard<std::mutex> g(mem_mu);
                if (!rc && ctx && I.n_forward > 0) {
                    uint64_t recs = 0;
                    for (int c = 0; c < ALB_CHANNELS; ++c) recs += ctx->h_rec_count[c];
                    rpp_seen = std::max(rpp_seen, (double)recs / (double)I.n_forward);
                }
                --running;
                mem_cv.notify_all();
            }
            I.status = rc;
            if (rc) {
                std::lock_guard<std::mutex> g(msg_mu);
                last_msg = msg;
                if (ctx && (rc == ALB_ERR_CUDA || rc == ALB_ERR_ITER_CAP || rc == ALB_ERR_CAPACITY)) {
                    alb_destroy(ctx);  // start the next instance clean
                    ctx = nullptr;
                }
                if (!ctx) {  // no context (destroyed, or never created): this worker holds nothing
                    std::lock_guard<std::mutex> m(mem_mu);
                    held_total -= held;
                    held = 0.0;
                    mem_cv.notify_all();
                }
            }
            // Device memory is admitted on an estimate: an instance that failed for memory
            // (an allocation or a map build) while others were running is run once more,
            // alone, once every other worker has released its context.
            const bool memory = rc == ALB_ERR_CUDA || rc == ALB_ERR_CAPACITY;
            const bool was_alone = alone;
            alone = memory && shared && !alone && cudaGetLastError() != cudaErrorIllegalAddress;
            if (alone || was_alone) {
                std::lock_guard<std::mutex> m(mem_mu);
                exclusive += alone ? 1 : -1;
                mem_cv.notify_all();
            }
        }
        if (ctx) alb_destroy(ctx);
        {
            std::lock_guard<std::mutex> g(mem_mu);
            held_total -= held;
            mem_cv.notify_all();
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (st) cudaStreamDestroy(st);
    };
    std::vector<std::thread> pool;
    const int K = (int)std::min<uint64_t>((uint64_t)opt->streams, std::max<uint64_t>(n, 1));
    for (int w = 0; w < K; ++w) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    g_create_error = last_msg;
    return ALB_OK;
}
