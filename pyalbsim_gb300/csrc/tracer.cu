// Tracer kernels: persistent grid-stride loop, one photon per thread at a time.
#include "device_common.cuh"
#include "internal.h"
#include "tracer.cuh"
#include "tracer_fast.cuh"

namespace alb {

constexpr int kTraceThreads = 128;

template <int PASS, bool REPLAY>
__global__ void __launch_bounds__(kTraceThreads) k_trace(SceneDev sc, TraceOut out, uint64_t n, uint64_t first,
                                                         uint32_t k0, uint32_t k1, const int64_t* __restrict__ offs,
                                                         const double* __restrict__ vals,
                                                         const float* __restrict__ taus) {
    unsigned long long events = 0, done = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t gid = first + i;
        const uint32_t pid = (uint32_t)gid;
        Ph ph;
        if (REPLAY) {
            ReplaySrc src{vals, taus, offs[i], offs[i + 1], out.err};
            emit_photon<PASS>(sc, ph, src);
            trace_photon<PASS>(sc, out, ph, src, pid, events);
        } else {
            PhiloxSrc src{k0, k1, (uint32_t)gid, (uint32_t)(gid >> 32), (uint32_t)PASS, 0u};
            emit_photon<PASS>(sc, ph, src);
            trace_photon<PASS>(sc, out, ph, src, pid, events);
        }
        if (out.ex_pos) {
            out.ex_pos[3 * i] = ph.px; out.ex_pos[3 * i + 1] = ph.py; out.ex_pos[3 * i + 2] = ph.pz;
            out.ex_dir[3 * i] = ph.dx; out.ex_dir[3 * i + 1] = ph.dy; out.ex_dir[3 * i + 2] = ph.dz;
            float* f = out.ex_f + 10 * i;
            f[0] = ph.E; f[1] = ph.tau; f[2] = ph.taut; f[3] = ph.t0;
            f[4] = ph.fwi[0]; f[5] = ph.fwi[1]; f[6] = ph.fwi[2];
            f[7] = ph.sfi[0]; f[8] = ph.sfi[1]; f[9] = ph.sfi[2];
        }
        ++done;
    }
    // warp-reduce the event counters, one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        events += __shfl_xor_sync(0xffffffffu, events, o);
        done += __shfl_xor_sync(0xffffffffu, done, o);
    }
    if ((threadIdx.x & 31) == 0 && out.stats) {
        atomicAdd(out.stats, events);
        atomicAdd(out.stats + 1, done);
    }
}

template <int PASS>
__global__ void __launch_bounds__(kTraceThreads) k_trace_fast(SceneDev sc, FastScene fs, TraceOut out, uint64_t n,
                                                              uint64_t first, uint32_t k0, uint32_t k1) {
    unsigned long long events = 0, done = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t gid = first + i;
        PhiloxSrc src{k0, k1, (uint32_t)gid, (uint32_t)(gid >> 32), (uint32_t)PASS, 0u};
        PhF ph;
        emit_photon_fast<PASS>(sc, ph, src);
        trace_photon_fast<PASS>(sc, fs, out, ph, src, (uint32_t)gid, events);
        if (out.ex_pos) {
            out.ex_pos[3 * i] = ph.px; out.ex_pos[3 * i + 1] = ph.py; out.ex_pos[3 * i + 2] = ph.pz;
            out.ex_dir[3 * i] = ph.dx; out.ex_dir[3 * i + 1] = ph.dy; out.ex_dir[3 * i + 2] = ph.dz;
            float* f = out.ex_f + 10 * i;
            f[0] = ph.E; f[1] = ph.tau; f[2] = ph.taut; f[3] = ph.t0;
            f[4] = ph.fwi[0]; f[5] = ph.fwi[1]; f[6] = ph.fwi[2];
            f[7] = ph.sfi[0]; f[8] = ph.sfi[1]; f[9] = ph.sfi[2];
        }
        ++done;
    }
    for (int o = 16; o > 0; o >>= 1) {
        events += __shfl_xor_sync(0xffffffffu, events, o);
        done += __shfl_xor_sync(0xffffffffu, done, o);
    }
    if ((threadIdx.x & 31) == 0 && out.stats) {
        atomicAdd(out.stats, events);
        atomicAdd(out.stats + 1, done);
    }
}

void launch_trace(const SceneDev& sc, const TraceOut& out, int pass, uint64_t n, uint64_t first_photon,
                  uint64_t seed, const AlbReplay* rp, int* launches, cudaStream_t st, const FastScene* fast) {
    if (n == 0) return;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t want = (n + kTraceThreads - 1) / kTraceThreads;
    uint64_t cap = (uint64_t)sms * 8;  // resident CTAs of the persistent grid
    unsigned blocks = (unsigned)(want < cap ? want : cap);
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    if (fast && !rp) {
        if (pass == ALB_FORWARD) k_trace_fast<ALB_FORWARD><<<blocks, kTraceThreads, 0, st>>>(sc, *fast, out, n, first_photon, k0, k1);
        else k_trace_fast<ALB_BACKWARD><<<blocks, kTraceThreads, 0, st>>>(sc, *fast, out, n, first_photon, k0, k1);
        note_launch();
        if (launches) ++*launches;
        return;
    }
    const int64_t* offs = rp ? rp->offsets : nullptr;
    const double* vals = rp ? rp->values : nullptr;
    const float* taus = rp ? rp->tau : nullptr;
    if (pass == ALB_FORWARD) {
        if (rp) k_trace<ALB_FORWARD, true><<<blocks, kTraceThreads, 0, st>>>(sc, out, n, first_photon, k0, k1, offs, vals, taus);
        else k_trace<ALB_FORWARD, false><<<blocks, kTraceThreads, 0, st>>>(sc, out, n, first_photon, k0, k1, offs, vals, taus);
    } else {
        if (rp) k_trace<ALB_BACKWARD, true><<<blocks, kTraceThreads, 0, st>>>(sc, out, n, first_photon, k0, k1, offs, vals, taus);
        else k_trace<ALB_BACKWARD, false><<<blocks, kTraceThreads, 0, st>>>(sc, out, n, first_photon, k0, k1, offs, vals, taus);
    }
    note_launch();
    if (launches) ++*launches;
}

}  // namespace alb
