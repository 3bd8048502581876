// alb_knn_noalloc: k-nearest-neighbour queries that allocate no device memory.
//
// Some callers of this library cannot call cudaMalloc: code running while a stream is
// being captured into a CUDA graph (a cudaMalloc there breaks the capture), a real-time
// acquisition loop that may only allocate at start-up, or a process whose device memory is
// owned by another framework's pool (a second allocator would exceed its budget). They
// already hold the input and output buffers; what they cannot provide is the index the
// query builds on the side. This entry point keeps that index in one file-scope static
// device array of fixed size, so it runs with the caller's buffers alone.
//
// Limits and sharing: at most ALB_NOALLOC_MAX_POINTS points per call (the k-d index of the
// points is built by one CTA in shared memory), k <= 256. Every call on a device uses the
// same static array and leaves its contents behind; each call rewrites every part it reads
// (the identity permutation, the cell descriptor, the index and its boxes) before use.
// Calls whose work overlaps on the GPU (different streams, or several host threads) race
// on the array and must be serialised by the caller.
//
// Set-up: the first call on a device looks the array's device address up with
// cudaGetSymbolAddress (with that device current) and sets the shared-memory limit of the
// build kernel; later calls reuse both. Make that first call before any stream capture.
#include <algorithm>
#include <mutex>
#include <string>

#include "albgpu.h"
#include "internal.h"

namespace alb {
int cell_index_max_points();
void launch_single_cell_index(const float4* pts, uint32_t n, const uint32_t* perm_in, const unsigned* cell,
                              uint32_t* perm_out, float4* sorted, float4* box_lo, float4* box_hi,
                              const uint64_t* lvl_off, const uint64_t* lvl_cnt, int nlevels, cudaStream_t st);
void set_global_error(const std::string& msg);
}  // namespace alb

using namespace alb;

namespace {

constexpr uint32_t kMaxPts = ALB_NOALLOC_MAX_POINTS;
constexpr uint32_t kMaxLeaves = kMaxPts / 32;
constexpr uint32_t kMaxBoxes = kMaxLeaves + kMaxLeaves / 32 + 2;

struct KnnScratch {
    float4 pts[kMaxPts];      // packed input points, w = original index
    float4 sorted[kMaxPts];   // k-d ordered copy (NaN dummies pad the last leaf)
    float4 box_lo[kMaxBoxes];
    float4 box_hi[kMaxBoxes];
    uint32_t perm_in[kMaxPts];
    uint32_t perm_out[kMaxPts];
    unsigned cell[4];         // start, count, padded start of the single cell
    int err;
};

// Modest by design: about 170 KB per device, held until the process exits.
static __device__ __align__(256) KnnScratch g_knn_scratch;

std::mutex g_setup_mutex;
KnnScratch* g_scratch_addr[64] = {nullptr};

__global__ void k_pack_points(const float* __restrict__ pts, uint32_t m, KnnScratch* s) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        s->pts[i] = make_float4(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], __uint_as_float(i));
        s->perm_in[i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s->cell[0] = 0u;
        s->cell[1] = m;
        s->cell[2] = 0u;
        s->err = 0;
    }
}

// neighbour positions in the k-d ordered copy -> the caller's point indices. A slot whose
// position is not one of the P slots of the ordered copy, or whose tag is not one of the m
// input points, is marked as failed (index -1, distance NaN) instead of being followed: the
// search writes -1 for a query it could not answer, and this call cannot synchronise to
// report the device-side status, so the marker is how a failure reaches the caller.
__global__ void k_map_tags(int32_t* idx, double* dist, uint64_t total, uint32_t P, uint32_t m, const KnnScratch* s) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t j = idx[i];
        uint32_t tag = 0xffffffffu;
        if (j >= 0 && (uint32_t)j < P) tag = __float_as_uint(s->sorted[j].w);
        if (tag < m) {
            idx[i] = (int32_t)tag;
        } else {
            idx[i] = -1;
            dist[i] = __longlong_as_double(0x7ff8000000000000ll);
        }
    }
}

KnnScratch* scratch_for_current_device() {
    int dev = 0;
    const cudaError_t ge = cudaGetDevice(&dev);
    if (ge != cudaSuccess) {
        set_global_error(std::string("alb_knn_noalloc: no usable current device: ") + cudaGetErrorString(ge));
        return nullptr;
    }
    if (dev < 0 || dev >= 64) {
        set_global_error("alb_knn_noalloc: current device " + std::to_string(dev) + " is outside the 64 supported");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_knn_scratch);
        if (e != cudaSuccess) {
            set_global_error(std::string("cudaGetSymbolAddress of the k-NN scratch failed: ") + cudaGetErrorString(e));
            return nullptr;
        }
        g_scratch_addr[dev] = (KnnScratch*)p;
    }
    return g_scratch_addr[dev];
}

}  // namespace

extern "C" int alb_knn_noalloc(const float* points_dev, uint64_t m, const double* queries_dev, uint64_t q, int k,
                               int32_t* idx_dev, double* dist_dev, void* stream) {
    if (!points_dev || !queries_dev || !idx_dev || !dist_dev) {
        set_global_error("alb_knn_noalloc: null buffer");
        return ALB_ERR_INVALID;
    }
    if (k < 1 || k > 256) {
        set_global_error("alb_knn_noalloc: k must be in [1, 256]");
        return ALB_ERR_INVALID;
    }
    if (m > kMaxPts || (uint64_t)cell_index_max_points() < m) {
        set_global_error("alb_knn_noalloc: at most " + std::to_string(kMaxPts) + " points per call (got " +
                         std::to_string(m) + ")");
        return ALB_ERR_INVALID;
    }
    if (m < (uint64_t)k) {
        set_global_error("alb_knn_noalloc: fewer points than k");
        return ALB_ERR_TOO_FEW;
    }
    if (q == 0) return ALB_OK;
    KnnScratch* s = scratch_for_current_device();
    if (!s) return ALB_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    // box tree shape of the padded point set
    const uint64_t P = (m + 31) / 32 * 32;
    uint64_t lvl_off[kMaxLevels] = {0}, lvl_cnt[kMaxLevels] = {0};
    uint64_t cnt = P / 32, off = 0;
    int nlevels = 0;
    while (true) {
        lvl_off[nlevels] = off;
        lvl_cnt[nlevels] = cnt;
        off += cnt;
        ++nlevels;
        if (cnt <= 32 || nlevels >= kMaxLevels) break;
        cnt = (cnt + 31) / 32;
    }
    k_pack_points<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(points_dev, (uint32_t)m, s);
    note_launch();
    launch_single_cell_index(s->pts, (uint32_t)m, s->perm_in, s->cell, s->perm_out, s->sorted, s->box_lo, s->box_hi,
                             lvl_off, lvl_cnt, nlevels, st);
    MapDev md{};
    md.a = s->sorted;
    md.b = s->sorted;  // the query path reads positions only
    md.box_lo = s->box_lo;
    md.box_hi = s->box_hi;
    md.n = P;
    md.n_real = m;
    md.nlevels = nlevels;
    for (int l = 0; l < kMaxLevels; ++l) {
        md.lvl_off[l] = lvl_off[l];
        md.lvl_cnt[l] = lvl_cnt[l];
    }
    launch_knn(md, queries_dev, q, k, idx_dev, dist_dev, &s->err, st);
    k_map_tags<<<(unsigned)std::min<uint64_t>((q * (uint64_t)k + 255) / 256, 65535), 256, 0, st>>>(
        idx_dev, dist_dev, q * (uint64_t)k, (uint32_t)P, (uint32_t)m, s);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_global_error(std::string("alb_knn_noalloc: launch failed: ") + cudaGetErrorString(e));
        return ALB_ERR_CUDA;
    }
    return ALB_OK;
}
