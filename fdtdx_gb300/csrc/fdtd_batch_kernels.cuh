// Batched (persistent) forms of the forward-step kernels: one launch per kernel kind runs
// the work of every simulation of a batch.  Each launch walks a flat list of work units
// (simulation, block of that simulation's launch) with a grid-stride loop; a unit runs the
// same device body the per-simulation kernel runs for that block, so results do not
// depend on batching.
#pragma once
#include "fdtd_kernels.cuh"

namespace fdtd {

// One block of one simulation's half-step launch.  Units are grouped by the kernel
// variant (z-vector width, CPML) of their part, one persistent launch per group, so each
// launch carries only its own variant's registers.
struct BUnit {
    int arg;   // index into the UpdArgs table (simulation part)
    int blk;   // block index within that launch
};

template <bool HSIDE, int VEC, bool PML>
__global__ void __launch_bounds__(256) k_batch_update(const BUnit* __restrict__ units, int n_units,
                                                      const UpdArgs* __restrict__ args) {
    for (int u = blockIdx.x; u < n_units; u += gridDim.x) {
        const BUnit bu = units[u];
        if (HSIDE) update_H_body<false, VEC, PML>(args[bu.arg], bu.blk);
        else update_E_body<false, VEC, PML>(args[bu.arg], bu.blk);
    }
}

// One source of one simulation (the field it injects into depends on the H parity).
struct BSrc {
    Geo g;
    DSource s;
    const int* tp;
    float* F[2];
    const float* mat;
    int n_mat;
    float mat_scalar;
};

template <bool ESIDE>
__global__ void __launch_bounds__(256) k_batch_source(const int2* __restrict__ units, int n_units,
                                                      const BSrc* __restrict__ args, int parity) {
    for (int u = blockIdx.x; u < n_units; u += gridDim.x) {
        const int2 bu = units[u];
        const BSrc& b = args[bu.x];
        source_body<ESIDE>(b.g, b.s, b.tp, b.F[parity], b.mat, b.n_mat, b.mat_scalar, 0, bu.y);
    }
}

// One non-fused detector of one simulation.
struct BDet {
    Geo g;
    DDet d;
    const int* tp;
    DetFields f[2];
    void* state;
};

__global__ void __launch_bounds__(kDetBlock) k_batch_detector(const int2* __restrict__ units, int n_units,
                                                              const BDet* __restrict__ args, int parity) {
    for (int u = blockIdx.x; u < n_units; u += gridDim.x) {
        const int2 bu = units[u];
        const BDet& b = args[bu.x];
        detector_body(b.g, b.d, b.tp, b.f[parity], b.state, bu.y);
    }
}

__global__ void __launch_bounds__(kDetBlock) k_batch_detector_finalize(const int* __restrict__ dets, int n,
                                                                       const BDet* __restrict__ args) {
    for (int u = blockIdx.x; u < n; u += gridDim.x) {
        const BDet& b = args[dets[u]];
        detector_finalize_body(b.d, b.tp, b.state);
    }
}

// PML-interface recording of one simulation (dtype per group).
struct BIface {
    Geo g;
    IfaceDev ifc;
    const int* tp;
    int n_slots;
    float* E;
    float* H[2];
    void* rec;
};

template <typename T>
__global__ void __launch_bounds__(256) k_batch_interfaces(const int2* __restrict__ units, int n_units,
                                                          const BIface* __restrict__ args, int parity) {
    for (int u = blockIdx.x; u < n_units; u += gridDim.x) {
        const int2 bu = units[u];
        const BIface& b = args[bu.x];
        interfaces_body<T, false>(b.g, b.ifc, b.tp, b.n_slots, b.E, b.H[parity], reinterpret_cast<T*>(b.rec), bu.y);
    }
}

__global__ void k_batch_advance(int* const* __restrict__ tps, int n) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) *tps[q] += 1;
}

}  // namespace fdtd
