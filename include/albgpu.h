/*
 * albgpu.h - C ABI of the GB300 photon-tracing / photon-mapping waveform engine.
 *
 * Plain pointers and sizes only. Host pointers are caller-owned; the context owns every
 * device buffer. Calls on one context are not re-entrant. All functions return ALB_OK (0)
 * or a negative ALB_ERR_* code; alb_last_error() gives the message of the last failure.
 *
 * Each entry point replaces one step of the reference's pure-Python driver
 * (alb_sim/execution/linear.py:77-117 run_linear, alb_sim/execution/parallel.py:186-284
 * run_parallel):
 *
 *   alb_create        Simulation(config, rng) + SimulationModel(config)
 *                     (alb_sim/core/simulation.py:29-69, physics/models/simulation.py:21-43)
 *   alb_trace pass 0  Simulation.simulate_batch(n, forward=True)
 *                     (core/simulation.py:71-107 with store_photons :113-130)
 *   alb_build_maps    build_photon_map_data + PhotonMapIndex(KDTree)
 *                     (photon_mapping/build_photon_map_data.py:8-62, photon_map_index.py:6-17)
 *   alb_trace pass 1  Simulation.simulate_batch(n, forward=False) including the k-NN
 *                     gathers and waveform accumulation (core/simulation.py:132-214)
 *   alb_get_waveform  Simulation.return_waveform[type] (core/simulation.py:46-49)
 *   alb_export_map    PhotonMapData of one type (photon_mapping/photon_map_data.py:6-15)
 *   alb_knn           KDTree(points).query(x, k) (photon_map_index.py:17,
 *                     core/simulation.py:139-142), exposed for neighbour-set checks
 */
#ifndef ALBGPU_H
#define ALBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ALB_MAX_LAYERS 8
#define ALB_PHASE_DIVISIONS 18000
#define ALB_CHANNELS 4

/* status codes */
#define ALB_OK 0
#define ALB_ERR_INVALID (-1)      /* bad argument or configuration (ValueError) */
#define ALB_ERR_TOO_FEW (-2)      /* photon map smaller than k at a gather (IndexError) */
#define ALB_ERR_CAPACITY (-3)     /* a device buffer bound was exceeded */
#define ALB_ERR_CUDA (-4)         /* CUDA runtime failure */
#define ALB_ERR_ITER_CAP (-5)     /* a device loop hit its iteration cap */
#define ALB_ERR_REPLAY (-6)       /* a replay stream ran out of variates */
#define ALB_ERR_STATE (-7)        /* call order violated (e.g. gather before maps) */

/* channels = PhotonType in the reference's enum order (photon_mapping/photon_type.py:7-10) */
#define ALB_BOTTOM_REFLECTION 0
#define ALB_SCATTER 1
#define ALB_SURFACE_REFLECTION 2
#define ALB_SURFACE_TRANSMISSION_UP 3

/* passes */
#define ALB_FORWARD 0
#define ALB_BACKWARD 1

/* options (alb_set_option) */
#define ALB_OPT_KEEP_EXIT_STATES 1 /* keep per-photon final states of the next trace */
#define ALB_OPT_KEEP_RECORD_IDS 2  /* store the emitting photon id with every record/query */
#define ALB_OPT_PRECISE 3          /* 1: float64 event geometry (replay-exact), 0: fast fp32 */
#define ALB_OPT_MAP_CAPACITY 4     /* records per channel to pre-allocate (0 = automatic) */
#define ALB_OPT_SORT_QUERIES 5     /* 1: sort gather queries spatially before the gather */
#define ALB_OPT_STREAM 6           /* cudaStream_t (as integer) used for every launch */
#define ALB_OPT_ADJOINT 7          /* 1: track path scores and accumulate d waveform / d theta
                                      (extension; set before the first forward trace of a
                                      simulation; constant layers only) */

/* One homogeneous water layer. The tables are host pointers read once by alb_create. */
typedef struct AlbLayer {
    double bottom_depth;          /* depth of the layer's lower boundary below the surface */
    double speed;                 /* c / n rounded to float32, m/s */
    float alpha;                  /* Churnside lidar attenuation (float32), 1/m */
    float ssa;                    /* single-scattering albedo (alpha - a) / alpha, float32 */
    double absorption;            /* absorption a, 1/m (adjoint only) */
    double bin_width;             /* angular bin width of the gather weight (float32 value) */
    const double* phase_theta;    /* ALB_PHASE_DIVISIONS scattering angles */
    const double* phase_cdf;      /* ALB_PHASE_DIVISIONS normalised CDF values */
    const double* phase_slope;    /* ALB_PHASE_DIVISIONS-1 interpolation slopes d theta/d cdf */
    const double* scatter_weight; /* ALB_PHASE_DIVISIONS CDF mass per angular bin */
    /* Depth profile (TurbidityLayerModel, alb_sim/physics/models/water.py:85-101,190-245).
     * profiled == 0: the constants above hold in the whole layer. Otherwise, at a local
     * depth z below the layer top, per integration step: speed = float32(c / n(z)),
     * attenuation = float32(interp(float32(z), lut_z, lut_alpha)), albedo =
     * float32((interp - a(z)) / interp). Profiles: kind 0 constant (start), 1 linear in
     * float32 (LinearParameter), 2 exponential in float64 (ExponentialParameter), at the
     * fraction z / height. */
    int32_t profiled;
    int32_t lut_n;                /* attenuation LUT entries (num_sublayers) */
    const float* lut_z;           /* linspace(0, height, lut_n) in float32 */
    const double* lut_alpha;      /* attenuation at lut_z */
    int32_t n_kind;               /* refractive index profile kind */
    int32_t a_kind;               /* absorption profile kind */
    double n_start, n_end;
    double a_start, a_end;
    double height;                /* layer thickness, m */
    double top32;                 /* depth of the layer top, rounded to float32 */
    /* Adjoint (extension, no counterpart in the reference). d ln(alpha)/d theta and
     * d ln(ssa)/d theta for theta = (a, b, g) of this layer, g the Henyey-Greenstein
     * asymmetry; hg_g != 0 marks an HG layer (its phase sampling and gather weight depend
     * on g); dlog_weight_g (ALB_PHASE_DIVISIONS, nullable) = d ln(scatter_weight)/dg.
     * dlog_sample_g (ALB_PHASE_DIVISIONS, nullable) = d ln(mass)/dg of each interval of the
     * sampling table, interval i holding the angles in (phase_theta[i-1], phase_theta[i]]
     * (i = 0: phase_theta[0]): the score of a drawn angle. NULL falls back to the analytic
     * d ln p_HG(mu)/dg, which is biased when the HG peak is narrow against the grid. */
    double dlog_alpha[3];
    double dlog_ssa[3];
    double hg_g;
    const double* dlog_weight_g;
    const double* dlog_sample_g;
} AlbLayer;

/* Scene constants derived on the host from SimulationConfig. */
typedef struct AlbSceneParams {
    double dt;                    /* integrator step, s */
    int64_t steps;                /* waveform samples of SimulationModel.steps; bins = 2*steps */
    int32_t sample_multiplier;    /* integrator steps per waveform sample */
    int32_t k;                    /* photon_mapping_k */
    double surface_y;             /* y of the mean water surface */
    double floor_y;               /* y of the seafloor */
    double speed_air;             /* float32-rounded speed of light in air */
    double n_water;               /* refractive index of the top layer at the surface */
    double f0;                    /* Schlick base reflectance */
    double seafloor_albedo;
    double surface_albedo;
    double roughness;             /* SeaSurfaceConfig.roughness (GGX alpha = roughness^2) */
    double laser_dir[3];
    float laser_rot[9];           /* float32 row-major rotation +z -> laser axis */
    double divergence;            /* beam half-angle, rad */
    double fov;                   /* receiver half-angle, rad */
    double aperture_radius;       /* m */
    double pulse_sigma;           /* s */
    double effective_rate;        /* sample_multiplier * sample_rate, Hz */
    int32_t n_layers;
    int32_t heatmap_enabled;
    int32_t heatmap_bins;
    int32_t reserved0;
    double heatmap_water_extent;
    double heatmap_floor_extent;
    double water_center[3];
    double floor_center[3];
    AlbLayer layers[ALB_MAX_LAYERS];
    /* Extension (no counterpart in the reference): > 0 selects the fixed-radius gather, every
     * record within this distance (m) with norm 1/(pi R^2) or 1/(4/3 pi R^3); 0 is k-NN. */
    double gather_radius;
    /* Extension: gated waveform window. gate_bins > 0 keeps bins [gate_start, gate_start +
     * gate_bins) of the 2*steps timeline (every waveform and Jacobian array then has
     * gate_bins entries) and drops contributions outside it; 0 keeps the whole timeline,
     * where a bin outside it is an error (ALB_ERR_CAPACITY). */
    int64_t gate_start;
    int64_t gate_bins;
    /* Extension: Gaussian surface slopes. > 0: at every surface interaction the facet normal
     * is normalize(-gx, 1, -gz), gx, gz ~ N(0, slope_sigma^2), for reflection, refraction and
     * Fresnel (Philox mode only); 0: the reference's flat surface. */
    double slope_sigma;
} AlbSceneParams;

/* Caller-supplied variates (replay mode): photon i consumes values[offsets[i] ..
 * offsets[i+1]) in the reference's draw order; tau[j] = -log(float32(values[j])) formed as
 * the reference forms it (used where a value is an optical-depth target). */
typedef struct AlbReplay {
    const int64_t* offsets;       /* n + 1 entries */
    const double* values;
    const float* tau;
    uint64_t n_values;
} AlbReplay;

typedef struct AlbCtx AlbCtx;

/* Simulation(config, rng): validate the scene, upload tables, allocate the context. */
int alb_create(const AlbSceneParams* scene, int device, AlbCtx** out);
void alb_destroy(AlbCtx* ctx);
const char* alb_last_error(const AlbCtx* ctx);
int alb_set_option(AlbCtx* ctx, int key, int64_t value);

/* simulate_batch(n, forward=pass==ALB_FORWARD). Philox mode when replay == NULL: photon i
 * of this call uses stream (seed, first_photon + i). Forward calls append records to the
 * photon maps; backward calls trace, gather and accumulate into the waveform. */
int alb_trace(AlbCtx* ctx, int pass, uint64_t n, uint64_t seed, uint64_t first_photon,
              const AlbReplay* replay);

/* build_photon_map_data + PhotonMapIndex: sort every channel's records into the spatial
 * index used by the gather. Must follow the forward traces and precede backward ones. */
int alb_build_maps(AlbCtx* ctx);

/* Records of one channel (after alb_build_maps: in index order). fwi/sfi (float[3n],
 * nullable) are the first-water / seafloor interaction points, stored only when the
 * scene's heatmaps are enabled (NaN otherwise), as PhotonMapData carries them. */
int alb_map_size(AlbCtx* ctx, int channel, uint64_t* out);
int alb_export_map(AlbCtx* ctx, int channel, float* pos, float* dir, float* energy,
                   float* time, float* fwi, float* sfi, int64_t* photon_id, size_t n);

/* Sampled heatmaps (alb_sim/math/accumulate_heatmap.py:6-124): water and seafloor energy
 * heatmaps (float64 [bins*bins]) and the forward scatter-radius counts (float32). */
int alb_get_heatmaps(AlbCtx* ctx, double* water, double* seafloor, float* radius, size_t bins2);

/* return_waveform[type] as float32 (reference units), or its exact float64 value. */
int alb_get_waveform(AlbCtx* ctx, int channel, float* out, size_t nbins);
int alb_get_waveform_f64(AlbCtx* ctx, int channel, double* out, size_t nbins);
int alb_reset_waveform(AlbCtx* ctx);

/* Start a new simulation on the same context: empty photon maps, queries, waveform and
 * heatmaps; device allocations are kept for reuse (a new Simulation(config, rng)). */
int alb_reset(AlbCtx* ctx);

/* Per-photon final states of the last trace (needs ALB_OPT_KEEP_EXIT_STATES):
 * pos/dir double[3n], energy/tau/tau_target/time float[n], fwi/sfi float[3n]. */
int alb_export_exit_states(AlbCtx* ctx, double* pos, double* dir, float* energy, float* tau,
                           float* tau_target, float* time, float* fwi, float* sfi, size_t n);

/* Backward queries of the last backward trace for one query kind (0 bottom, 1 scatter,
 * 2 surface): pos double[3n], dir float[3n], energy/time float[n], photon ids, k-th
 * neighbour distance r_k double[n] per map gathered (surface queries gather twice:
 * rk2 is the transmission map's, NULL allowed). */
int alb_query_count(AlbCtx* ctx, int kind, uint64_t* out);
int alb_export_queries(AlbCtx* ctx, int kind, double* pos, float* dir, float* energy,
                       float* time, int64_t* photon_id, double* rk, double* rk2, size_t n);

/* KDTree(points).query(queries, k): exact k nearest neighbours on the device.
 * points float[3m] host, queries double[3q] host; out idx int32[q*k] sorted by distance,
 * dist double[q*k]. */
int alb_knn(AlbCtx* ctx, const float* points, uint64_t m, const double* queries, uint64_t q,
            int k, int32_t* idx, double* dist);

/* KDTree(points).query(queries, k) that allocates no device memory. It has no counterpart
 * in the reference: it exists for callers that cannot call cudaMalloc (code running during
 * a CUDA-graph stream capture, real-time loops that allocate only at start-up, processes
 * whose device memory belongs to another framework's pool). All buffers are DEVICE
 * pointers owned by the caller: points float[3m], queries double[3q], idx int32[q*k]
 * (nearest first), dist double[q*k]; stream is a cudaStream_t (NULL = legacy default).
 * The k-d index is built in a fixed static device array: m <= ALB_NOALLOC_MAX_POINTS,
 * k <= 256, larger inputs are rejected with ALB_ERR_INVALID. The first call on a device
 * resolves the array's address (make it before any stream capture); calls that overlap
 * on the GPU share the array and race. Asynchronous on `stream`; the message of a failed
 * call is alb_last_error(NULL). The call returns before the GPU has run, so a query the
 * search could not answer (NaN or infinite coordinates, or a traversal that hit its
 * iteration cap) is reported in the output instead: all k of its slots hold index -1 and
 * distance NaN. */
#define ALB_NOALLOC_MAX_POINTS 4096
int alb_knn_noalloc(const float* points_dev, uint64_t m, const double* queries_dev, uint64_t q, int k,
                    int32_t* idx_dev, double* dist_dev, void* stream);

/* Adjoint (extension, no counterpart in the reference), enabled by ALB_OPT_ADJOINT.
 * Parameters: 0 water depth, 1 absorption a, 2 scattering b, 3 HG asymmetry g, 4 seafloor
 * albedo, 5 surface roughness (a, b and g move every layer together). Every record and
 * query carries the score d ln(p E)/d theta of its path prefix (theta = a, b, g, albedo);
 * the gather adds c (s_query + s_record + d ln w/d theta) per neighbour into a Jacobian
 * held like the waveform (128-bit fixed point). The depth moves the seafloor plane and
 * with it the discrete return step, which has no score form; the host forms that column by
 * a central difference with common random numbers, so parameter 0 is rejected here.
 * alb_get_jacobian: d waveform[channel] / d theta[param] (float64 [nbins]).
 * alb_adjoint: grad[p] = sum over channels and bins of dL_dw[c][b] * J[p][c][b] for
 * p = 1..5 (dL_dw is float64 [ALB_CHANNELS][nbins]); grad[0] is set to NaN.
 * alb_export_map_scores: the per-record scores (float[4n]: a, b, g, albedo), in the order
 * of alb_export_map. */
#define ALB_ADJ_PARAMS 6
int alb_get_jacobian(AlbCtx* ctx, int param, int channel, double* out, size_t nbins);
int alb_adjoint(AlbCtx* ctx, const double* dL_dw, size_t nbins, double* grad);
int alb_export_map_scores(AlbCtx* ctx, int channel, float* scores, size_t n);

/* Batched instances (extension: the reference runs one configuration per process; its
 * hypercube notebook loops run_parallel over samples). Each instance is a full simulation:
 * n_forward photons traced into fresh photon maps, the maps indexed, n_backward photons
 * traced and gathered (Philox streams keyed by seed, photon ids from 0). `streams` host
 * workers each own a context on its own non-blocking CUDA stream and take instances from a
 * shared queue, largest (n_forward + n_backward) first, so small instances overlap on the
 * GPU; a context keeps its device buffers from one instance to the next. Device memory is
 * admitted on an estimate of each instance's footprint; an instance that fails for device
 * memory while others were running is run once more alone, after every other worker has
 * released its buffers. Results: the
 * float64 waveform [ALB_CHANNELS][2*steps] of each instance and, with adjoint set, its
 * Jacobian [ALB_ADJ_PARAMS-1][ALB_CHANNELS][2*steps] (parameters 1..5; nullable). The
 * call returns ALB_OK once every instance has run; each instance's own result is in
 * status (its message in alb_last_error(NULL) when it is the last failure). */
typedef struct AlbBatchInstance {
    const AlbSceneParams* scene;
    uint64_t n_forward;
    uint64_t n_backward;
    uint64_t seed;
    double* waveform;             /* out, caller-owned host memory */
    double* jacobian;             /* out (adjoint), nullable: NULL runs the instance plain */
    int32_t status;               /* out: ALB_OK or the instance's error code */
    float device_ms;              /* out: CUDA-event time of the instance on its stream */
} AlbBatchInstance;

typedef struct AlbBatchOptions {
    int32_t device;
    int32_t streams;              /* concurrent workers, 1..64 */
    int32_t precise;              /* 1: float64-geometry tracer, 0: fast float32 tracer */
    int32_t adjoint;              /* 1: also accumulate the Jacobian */
} AlbBatchOptions;

int alb_batch_run(AlbBatchInstance* instances, uint64_t n, const AlbBatchOptions* options);

/* Device-side counters: [0] events and [1] photons of the last trace, [2] kernels launched
 * by this library, [4 + 4c .. 7 + 4c] gather counters of channel c (leaves, nodes, selects,
 * queries), [24 + c] inexact queries of channel c, [28] events and [29] photons of the last
 * forward trace, [30] neighbour searches of the last trace redone because their first,
 * guessed threshold did not hold. n entries are written (at most 32). */
int alb_stats(AlbCtx* ctx, int64_t* out, int n);

/* Accumulated device time (ms, CUDA events on the context's stream) and call counts per
 * phase since the last reset: 0 forward trace, 1 map build, 2 backward trace,
 * 3 query sort, 4..7 gather of channel 0..3. out_ms/out_calls hold ALB_PHASES entries;
 * gathers[4] (nullable) receives the number of queries gathered per channel.
 * reset != 0 clears the accumulators after reading. */
#define ALB_PHASES 8
int alb_phase_times(AlbCtx* ctx, double* out_ms, int64_t* out_calls, int64_t* gathers, int reset);

#ifdef __cplusplus
}
#endif
#endif /* ALBGPU_H */
