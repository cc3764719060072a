// The tables of one persistent batch launch (fdtd_fused.cu), shared by the launching
// translation unit and the one that compiles the persistent kernel.  Plain device pointers:
// the kernel side reads them with the batch table types of fdtd_batch_kernels.cuh.
#pragma once
#include <cstdint>

struct FdtdFusedTables {
    const void* units;      // BUnit[n_units], grouped by update class
    int n_units;
    int class_start[5];     // unit ranges of the (vec, pml) classes (1,0) (1,1) (2,0) (2,1)
    const void* argsE;      // UpdArgs[2][max_args] (by H parity)
    const void* argsH;
    int max_args;
    const void* src_unitsE; // int2[n_src_unitsE]
    int n_src_unitsE;
    const void* srcE;       // BSrc[]
    const void* src_unitsH;
    int n_src_unitsH;
    const void* srcH;
    const void* iface_units;  // int2[], grouped by recording dtype
    int iface_start[4];
    const void* ifaces;       // BIface[]
    const void* det_units;    // int2[n_det_units]
    int n_det_units;
    const void* dets;         // BDet[]
    const int* det_red;       // reducing detectors
    int n_det_red;
    int* const* tps;          // step counter of each simulation
    int n_sims;
    int any_hprev;
    unsigned* bar;            // grid barrier: arrival count, generation
    int* err;                 // FDTD_ETIMEOUT when a barrier wait ran out
    long long spin_limit;     // iterations a barrier wait may spin
    int inject_skip;          // failure injection: block 0 never arrives at the first barrier
};

// Runs `steps` batch steps from H parity `parity` in one cooperative launch on `stream`
// with as many resident blocks as the device holds; returns 0, or the CUDA error code.
extern "C" int fdtd_fused_launch(const FdtdFusedTables* t, int steps, int parity, void* stream);
