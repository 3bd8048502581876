// Internal declarations shared by the translation units of libalbgpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "albgpu.h"
#include "device_common.cuh"
#include "tracer.cuh"

namespace alb {

constexpr int kMaxLevels = 8;
// Jacobian columns formed on the device: a, b, g, albedo, roughness (the depth column is a
// host-side difference)
constexpr int kJacParams = ALB_ADJ_PARAMS - 1;

// Number of kernels this library has launched (all contexts); read by alb_stats.
long long launches_total();
void note_launch();

// Uniform key grid over a bounding box; axes with no extent carry no key bits.
struct KeyGrid {
    double lo[3];
    double scale[3];
    double maxq[3];
    int ax[3];
    int naxes;
};

// Unsorted records of one channel as appended by the forward tracer.
// The two halves of a record are interleaved in one allocation owned by `a`: record r is
// a[2 r] = (x, y, z, energy) and b[2 r] = a[2 r + 1] = (dx, dy, dz, time), so a record is one
// aligned 32-byte sector (written once by the tracer, gathered once by the index build).
struct RecordStore {
    float4* a = nullptr;    // x, y, z, energy (stride 2)
    float4* b = nullptr;    // dx, dy, dz, time (stride 2; a + 1, not a separate allocation)
    float4* fwi = nullptr;  // optional
    float4* sfi = nullptr;
    uint32_t* id = nullptr; // optional
    float4* sco = nullptr;  // adjoint path scores (a, b, g, albedo), optional
    uint64_t cap = 0;
};

// Sorted records + implicit 32-ary box tree of one channel.
struct MapIndex {
    uint64_t n = 0;       // records in the index, including padding dummies
    uint64_t n_real = 0;  // records of the photon map
    float4* a = nullptr;
    float4* b = nullptr;
    float4* fwi = nullptr;
    float4* sfi = nullptr;
    uint32_t* id = nullptr;
    float4* sco = nullptr;
    uint64_t a_cap = 0, b_cap = 0, fwi_cap = 0, sfi_cap = 0, id_cap = 0, sco_cap = 0;
    float4* box_lo = nullptr;
    float4* box_hi = nullptr;
    uint64_t box_cap = 0, box_cap_hi = 0, nboxes = 0;
    int nlevels = 0;
    uint64_t lvl_off[kMaxLevels] = {0};
    uint64_t lvl_cnt[kMaxLevels] = {0};
};

// Device view of a map for the gather kernels.
struct MapDev {
    const float4* a;
    const float4* b;
    const float4* fwi;
    const float4* sfi;
    const float4* sco;  // adjoint path scores (nullable)
    const float4* box_lo;
    const float4* box_hi;
    uint64_t n;
    uint64_t n_real;
    int nlevels;
    uint64_t lvl_off[kMaxLevels];
    uint64_t lvl_cnt[kMaxLevels];
};

// Device view of one kind of gather queries.
struct QueryDev {
    const float4* a;   // x_hi, y_hi, z_hi, energy
    const float4* b;   // dx, dy, dz, time
    const float4* c;   // x_lo, y_lo, z_lo
    const float4* s;   // adjoint path scores (a, b, g, albedo), nullable
    const uint32_t* perm;  // optional processing order
    uint64_t n;
    double* rk_out;    // optional per-query k-th neighbour distance
    unsigned long long* stats;    // optional [leaves, nodes, selects, queries] accumulators
    unsigned long long* inexact;  // optional count of answers a buffer bound made inexact (mass ties)
    unsigned long long* retries;  // optional count of searches redone because a first guess did not hold
};

// Waveform / heatmap accumulators (128-bit fixed point, lo and hi words).
struct Accum {
    unsigned long long* wf_lo;  // [channels][nbins]
    unsigned long long* wf_hi;
    unsigned long long* hw_lo;  // sampled water heatmap [bins*bins] (nullable)
    unsigned long long* hw_hi;
    unsigned long long* hf_lo;  // sampled seafloor heatmap
    unsigned long long* hf_hi;
    int64_t nbins;
    unsigned long long* jac_lo;  // adjoint [5 params][channels][nbins] (nullable)
    unsigned long long* jac_hi;
};

// Stream-ordered device memory: temporaries come from cudaMallocAsync and are released in
// stack order; persistent buffers grow on demand.
class Workspace {
  public:
    explicit Workspace(cudaStream_t st = 0) : st_(st) {}
    ~Workspace();
    void set_stream(cudaStream_t st) { st_ = st; }
    void* take_bytes(uint64_t bytes);
    uint32_t* take_u32(uint64_t n) { return (uint32_t*)take_bytes(n * sizeof(uint32_t)); }
    size_t mark() const { return temps_.size(); }
    void release(size_t m);
    unsigned* scratch_box();
    void* alloc_persistent(void* old, uint64_t& cap, uint64_t n_float4);
    void* alloc_persistent_u32(void* old, uint64_t& cap, uint64_t n);
    bool failed() const { return failed_; }
    void clear_failed() { failed_ = false; }

  private:
    cudaStream_t st_;
    std::vector<void*> temps_;
    unsigned* box_ = nullptr;
    bool failed_ = false;
};

// ---- map build (mapbuild.cu)
KeyGrid make_key_grid(const float lo[3], const float hi[3], int bits3, int bits2);
int compute_bbox(Workspace& ws, const float4* a, uint64_t n, float lo[3], float hi[3], cudaStream_t st,
                 uint64_t stride = 1);
int build_map_index(Workspace& ws, const RecordStore& rec, uint64_t n, MapIndex& m, cudaStream_t st);
void release_map_index(MapIndex& m);
int build_box_tree(Workspace& ws, MapIndex& m, cudaStream_t st);
int sort_queries(Workspace& ws, const float4* qa, uint64_t n, uint32_t* perm, cudaStream_t st);

// ---- tracer (tracer.cu)
struct FastScene;
void launch_trace(const SceneDev& sc, const TraceOut& out, int pass, uint64_t n, uint64_t first_photon,
                  uint64_t seed, const AlbReplay* replay_dev, int* launches, cudaStream_t st,
                  const FastScene* fast);

// ---- gather (gather.cu)
void launch_gather(const SceneDev& sc, const MapDev& map, const QueryDev& q, int channel, const Accum& acc,
                   int* err, int* launches, cudaStream_t st);
void launch_knn(const MapDev& map, const double* queries, uint64_t nq, int k, int32_t* out_idx,
                double* out_dist, int* err, cudaStream_t st);

inline MapDev map_dev(const MapIndex& m) {
    MapDev d{};
    d.a = m.a;
    d.b = m.b;
    d.fwi = m.fwi;
    d.sfi = m.sfi;
    d.sco = m.sco;
    d.box_lo = m.box_lo;
    d.box_hi = m.box_hi;
    d.n = m.n;
    d.n_real = m.n_real;
    d.nlevels = m.nlevels;
    for (int i = 0; i < kMaxLevels; ++i) {
        d.lvl_off[i] = m.lvl_off[i];
        d.lvl_cnt[i] = m.lvl_cnt[i];
    }
    return d;
}

}  // namespace alb
