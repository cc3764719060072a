// One persistent launch for many steps of a whole batch (sm_103a): every block walks the
// batch's work units phase by phase -- E half-step, E sources, H half-step (with the fused
// detectors), H sources, interface recording and detectors, detector reductions, step
// counters -- with a grid-wide barrier between phases, for all the requested steps.  The
// phase bodies are the per-simulation kernels' device bodies, so results equal the other
// batch modes.  The launch is cooperative (every block resident), each barrier wait is
// bounded (an expired wait sets FDTD_ETIMEOUT and the kernel returns), and no load of data
// the launch writes takes the read-only path (FDTD_COHERENT_LOADS): plain loads after the
// barrier's release / acquire fences see every block's writes of the earlier phases.
#include <cuda_runtime.h>

#define FDTD_COHERENT_LOADS 1
#define fdtd fdtd_coh
#include "fdtd_batch_kernels.cuh"
#undef fdtd
#include "fdtd_fused.h"

namespace fdtd_coh {

// Grid-wide barrier over a cooperative launch: an arrival count and a generation word.  The
// last block to arrive resets the count and advances the generation; the others wait for the
// generation to change, at most `limit` polls, then set the error word and give up.
__device__ __forceinline__ bool grid_sync(unsigned* bar, int* err, long long limit) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long it = 0;
            while (*vgen == gen) {
                if (++it > limit || *(volatile int*)err) {
                    atomicCAS(err, 0, FDTD_ETIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// The phases and the per-unit bodies, each a separate (not inlined) function: the persistent
// kernel then needs only the registers of its largest piece, not of all of them at once.
// Each unit's table entry is passed as a __restrict__ pointer, so the compiler may keep the
// entry's fields in registers across the body's stores to the fields (as the persistent-mode
// kernels, whose table pointers are __restrict__ kernel parameters, do).
template <bool HSIDE, int VEC, bool PML>
__device__ __noinline__ void unit_update(const UpdArgs* __restrict__ a, int blk) {
    if (HSIDE) update_H_body<false, VEC, PML>(*a, blk);
    else update_E_body<false, VEC, PML>(*a, blk);
}

template <bool HSIDE>
__device__ __noinline__ void phase_update(const FdtdFusedTables& t, int parity) {
    const BUnit* __restrict__ units = static_cast<const BUnit*>(t.units);
    const UpdArgs* __restrict__ args = static_cast<const UpdArgs*>(HSIDE ? t.argsH : t.argsE) + parity * t.max_args;
    const int n = t.n_units, c1 = t.class_start[1], c2 = t.class_start[2], c3 = t.class_start[3];
    for (int u = blockIdx.x; u < n; u += gridDim.x) {
        const BUnit bu = units[u];
        if (u < c1) unit_update<HSIDE, 1, false>(args + bu.arg, bu.blk);
        else if (u < c2) unit_update<HSIDE, 1, true>(args + bu.arg, bu.blk);
        else if (u < c3) unit_update<HSIDE, 2, false>(args + bu.arg, bu.blk);
        else unit_update<HSIDE, 2, true>(args + bu.arg, bu.blk);
    }
}

template <bool ESIDE>
__device__ __noinline__ void unit_source(const BSrc* __restrict__ b, int parity, int blk) {
    source_body<ESIDE>(b->g, b->s, b->tp, b->F[parity], b->mat, b->n_mat, b->mat_scalar, 0, blk);
}

template <bool ESIDE>
__device__ __noinline__ void phase_sources(const FdtdFusedTables& t, int parity) {
    const int2* __restrict__ su = static_cast<const int2*>(ESIDE ? t.src_unitsE : t.src_unitsH);
    const BSrc* __restrict__ src = static_cast<const BSrc*>(ESIDE ? t.srcE : t.srcH);
    const int n = ESIDE ? t.n_src_unitsE : t.n_src_unitsH;
    for (int u = blockIdx.x; u < n; u += gridDim.x) {
        const int2 bu = su[u];
        unit_source<ESIDE>(src + bu.x, parity, bu.y);
    }
}

template <typename T>
__device__ __noinline__ void unit_interfaces(const BIface* __restrict__ b, int parity, int blk) {
    interfaces_body<T, false>(b->g, b->ifc, b->tp, b->n_slots, b->E, b->H[parity], static_cast<T*>(b->rec), blk);
}

__device__ __noinline__ void unit_detector(const BDet* __restrict__ b, int parity, int blk) {
    detector_body(b->g, b->d, b->tp, b->f[parity], b->state, blk);
}

__device__ __noinline__ void phase_record_and_detect(const FdtdFusedTables& t, int parity) {
    const int2* __restrict__ iu = static_cast<const int2*>(t.iface_units);
    const BIface* __restrict__ ifs = static_cast<const BIface*>(t.ifaces);
    const int i1 = t.iface_start[1], i2 = t.iface_start[2], i3 = t.iface_start[3];
    for (int u = blockIdx.x; u < i3; u += gridDim.x) {
        const int2 bu = iu[u];
        if (u < i1) unit_interfaces<float>(ifs + bu.x, parity, bu.y);
        else if (u < i2) unit_interfaces<__nv_bfloat16>(ifs + bu.x, parity, bu.y);
        else unit_interfaces<__half>(ifs + bu.x, parity, bu.y);
    }
    const int2* __restrict__ du = static_cast<const int2*>(t.det_units);
    const BDet* __restrict__ dets = static_cast<const BDet*>(t.dets);
    const int nd = t.n_det_units;
    for (int u = blockIdx.x; u < nd; u += gridDim.x) {
        const int2 bu = du[u];
        unit_detector(dets + bu.x, parity, bu.y);
    }
}

__device__ __noinline__ void unit_reduce(const BDet* __restrict__ b) { detector_finalize_body(b->d, b->tp, b->state); }

__device__ __noinline__ void phase_reduce(const FdtdFusedTables& t) {
    const BDet* __restrict__ dets = static_cast<const BDet*>(t.dets);
    const int* __restrict__ red = t.det_red;
    const int n = t.n_det_red;
    for (int u = blockIdx.x; u < n; u += gridDim.x) unit_reduce(dets + red[u]);
}

// Failure injection (tests only): a block that never arrives.  It waits, bounded, for the
// others' barrier wait to run out and report it, then leaves; every block ends.
__device__ __noinline__ void absent_block(const FdtdFusedTables& t) {
    if (threadIdx.x == 0) {
        long long it = 0;
        while (!*(volatile int*)t.err && ++it <= t.spin_limit) __nanosleep(64);
        atomicCAS(t.err, 0, FDTD_ETIMEOUT);
    }
    __syncthreads();
}

// Four resident blocks per SM (64 registers a thread): the memory-bound update phases need
// the warps more than the CPML H variants need the registers they then spill (measured on
// 64-simulation batches against two and three blocks).
#ifndef FDTD_FUSED_MIN_BLOCKS
#define FDTD_FUSED_MIN_BLOCKS 4
#endif

__global__ void __launch_bounds__(256, FDTD_FUSED_MIN_BLOCKS) k_batch_fused(const __grid_constant__ FdtdFusedTables t, int steps, int parity) {
    for (int s = 0; s < steps; ++s) {
        phase_update<false>(t, parity);
        if (t.inject_skip && s == 0 && blockIdx.x == 0) {
            absent_block(t);
            return;
        }
        if (!grid_sync(t.bar, t.err, t.spin_limit)) return;
        phase_sources<true>(t, parity);
        if (!grid_sync(t.bar, t.err, t.spin_limit)) return;
        phase_update<true>(t, parity);
        if (!grid_sync(t.bar, t.err, t.spin_limit)) return;
        phase_sources<false>(t, parity);
        if (!grid_sync(t.bar, t.err, t.spin_limit)) return;
        phase_record_and_detect(t, parity);
        if (!grid_sync(t.bar, t.err, t.spin_limit)) return;
        phase_reduce(t);
        if (!grid_sync(t.bar, t.err, t.spin_limit)) return;
        if (blockIdx.x == 0)
            for (int q = threadIdx.x; q < t.n_sims; q += blockDim.x) atomicAdd(t.tps[q], 1);
        if (!grid_sync(t.bar, t.err, t.spin_limit)) return;
        parity ^= t.any_hprev;
    }
}

}  // namespace fdtd_coh

extern "C" int fdtd_fused_launch(const FdtdFusedTables* t, int steps, int parity, void* stream) {
    int dev = 0, sms = 0, occ = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return (int)cudaErrorInvalidDevice;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fdtd_coh::k_batch_fused, 256, 0);
    if (e != cudaSuccess) return (int)e;
    if (!coop || occ <= 0 || sms <= 0) return (int)cudaErrorCooperativeLaunchTooLarge;
    FdtdFusedTables tt = *t;
    void* args[] = {&tt, &steps, &parity};
    e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(fdtd_coh::k_batch_fused), dim3(occ * sms), dim3(256),
                                    args, 0, reinterpret_cast<cudaStream_t>(stream));
    return (int)e;
}
