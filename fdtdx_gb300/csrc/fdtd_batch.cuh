// Host side of the batched forward path (fdtd_batch_*; included by fdtd_plan.cu, which owns
// the plan type and the launch helpers).
//
// A batch holds already-built plans and their buffers.  One batch step runs, for every
// simulation at once: the E half-step (core and CPML shell of every simulation in one
// persistent launch), the E-side sources, the H half-step with the fused detectors, the
// H-side sources, the remaining detectors (+ their reductions) and the step counters:
// five to six launches per step for the whole batch instead of about eight per
// simulation.  The step loop is captured in a CUDA graph.  Tile shapes (x planes per core
// unit, per shell unit, resident blocks per SM) are chosen by an online autotuner that
// times candidates on real steps of the batch (they change the work partition only, not
// the arithmetic), so tuning costs no extra simulation work.
#pragma once
#include "fdtd_batch_kernels.cuh"
#include "fdtd_fused.h"

struct FdtdBatch {
    int n = 0;
    std::vector<FdtdPlan*> plans;
    std::vector<FdtdBuffers> bufs;
    std::vector<int> t;                  // current step of each simulation (host mirror)
    bool any_hprev = false;
    int sm_count = 1;
    // tuning
    int chunk_scale_num = 1, chunk_scale_den = 1;  // core x-chunk = default chunk * num / den
    int shell_chunk = kShellChunk;
    int blocks_per_sm = 8;
    bool tuned = false;
    // device tables
    char* dmem = nullptr;
    UpdArgs* argsE = nullptr;  // [2 parities][n_args]
    UpdArgs* argsH = nullptr;
    BUnit* units = nullptr;
    int class_start[5] = {0, 0, 0, 0, 0};  // unit ranges of the (vec, pml) classes: (1,0) (1,1) (2,0) (2,1)
    BSrc* srcE = nullptr;
    BSrc* srcH = nullptr;
    int2* src_unitsE = nullptr;
    int2* src_unitsH = nullptr;
    BDet* dets = nullptr;
    int2* det_units = nullptr;
    int* det_red = nullptr;
    BIface* ifaces = nullptr;
    int2* iface_units = nullptr;
    int iface_start[4] = {0, 0, 0, 0};  // unit ranges per recording dtype (float, bf16, half)
    int** tps = nullptr;
    int n_args = 0, n_units = 0, n_srcE = 0, n_srcH = 0, n_src_unitsE = 0, n_src_unitsH = 0;
    int n_dets = 0, n_det_units = 0, n_det_red = 0;
    int max_args = 0, max_units = 0;
    // graph of a fixed number of steps
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    int gsteps = 0;
    cudaStream_t cap_stream = nullptr;
    // mode 1 ("branches"): each simulation's own launch chain (TMA cores) on its own stream,
    // forked from and joined to the caller's stream -- parallel branches of one graph
    // mode 2 ("fused"): all steps of a call in one cooperative launch (fdtd_fused.cu) with a
    // bounded grid barrier between phases; fbar / ferr are its barrier and error words
    int mode = 0;
    unsigned* fbar = nullptr;
    int* ferr = nullptr;
    mutable int fused_rc = 0;
    std::vector<cudaStream_t> sim_streams;
    std::vector<cudaEvent_t> join_ev;
    cudaEvent_t fork_ev = nullptr;
    std::string err;
};

namespace {

int bfail(FdtdBatch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

void batch_drop_graph(FdtdBatch* b) {
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    b->gsteps = 0;
}

int scaled_chunk(const FdtdBatch* b, const FdtdPlan* p) {
    return std::max(1, p->chunk * b->chunk_scale_num / b->chunk_scale_den);
}

// The update parts of one simulation: (box list, chunk per box, pml) for the core and the
// shell, or one CPML part over the whole grid.
struct BPart {
    Box boxes[6];
    int chunks[6];
    int n;
    bool pml;
};

int sim_parts(const FdtdBatch* b, const FdtdPlan* p, BPart parts[2]) {
    const Split sp = split_boxes(p);
    if (!sp.split) {
        parts[0].boxes[0] = Box{{0, 0, 0}, {p->g.nx, p->g.ny, p->g.nz}};
        parts[0].chunks[0] = scaled_chunk(b, p);
        parts[0].n = 1;
        parts[0].pml = true;
        return 1;
    }
    parts[0].boxes[0] = sp.core;
    parts[0].chunks[0] = scaled_chunk(b, p);
    parts[0].n = 1;
    parts[0].pml = false;
    if (sp.n_shell == 0) return 1;
    for (int q = 0; q < sp.n_shell; ++q) {
        parts[1].boxes[q] = sp.shell[q];
        parts[1].chunks[q] = b->shell_chunk;
    }
    parts[1].n = sp.n_shell;
    parts[1].pml = true;
    return 2;
}

// Rebuilds the update tables and the unit list for the current tile choice and uploads them.
int batch_build_updates(FdtdBatch* b) {
    // the tables may be read by steps still in flight on any stream
    cudaError_t se = cudaDeviceSynchronize();
    if (se != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("batch rebuild: ") + cudaGetErrorString(se));
    std::vector<BUnit> units, cunits[4];
    std::vector<UpdArgs> e0, e1, h0, h1;
    for (int s = 0; s < b->n; ++s) {
        FdtdPlan* p = b->plans[s];
        const FdtdBuffers* bb = &b->bufs[s];
        float* hc[2] = {bb->H, p->need_hprev ? p->h_twin : bb->H};
        float* hn[2] = {p->need_hprev ? p->h_twin : bb->H, bb->H};
        BPart parts[2];
        const int np = sim_parts(b, p, parts);
        for (int q = 0; q < np; ++q) {
            UpdArgs ae[2], ah[2];
            long long blocks = 0;
            for (int par = 0; par < 2; ++par) {
                ae[par] = make_upd(p, bb, true, hc[par], bb->E, bb->E);
                ah[par] = make_upd_fwd_H(p, bb, hc[par], hn[par]);
                ae[par].chunk = ah[par].chunk = parts[q].chunks[0];
                blocks = fill_boxes(p, ae[par], parts[q].boxes, parts[q].chunks, parts[q].n);
                fill_boxes(p, ah[par], parts[q].boxes, parts[q].chunks, parts[q].n);
            }
            const int arg = (int)e0.size();
            e0.push_back(ae[0]); e1.push_back(ae[1]);
            h0.push_back(ah[0]); h1.push_back(ah[1]);
            const int cls = (p->vec == 2 ? 2 : 0) + (parts[q].pml ? 1 : 0);
            for (long long k = 0; k < blocks; ++k) cunits[cls].push_back(BUnit{arg, (int)k});
        }
    }
    for (int cls = 0; cls < 4; ++cls) {
        b->class_start[cls] = (int)units.size();
        units.insert(units.end(), cunits[cls].begin(), cunits[cls].end());
    }
    b->class_start[4] = (int)units.size();
    b->n_args = (int)e0.size();
    b->n_units = (int)units.size();
    if (b->n_args > b->max_args || b->n_units > b->max_units) return bfail(b, FDTD_EINVAL, "batch tables overflow");
    // parity tables are laid out [parity * max_args + arg]
    cudaError_t e = cudaMemcpy(b->argsE, e0.data(), sizeof(UpdArgs) * b->n_args, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->argsE + b->max_args, e1.data(), sizeof(UpdArgs) * b->n_args, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->argsH, h0.data(), sizeof(UpdArgs) * b->n_args, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->argsH + b->max_args, h1.data(), sizeof(UpdArgs) * b->n_args, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->units, units.data(), sizeof(BUnit) * b->n_units, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("batch table upload: ") + cudaGetErrorString(e));
    batch_drop_graph(b);
    return FDTD_OK;
}

long long sim_update_blocks_upper(const FdtdPlan* p) {
    // blocks of the finest tiling the tuner may choose (chunk 1): an upper bound for the tables
    const Split sp = split_boxes(p);
    auto blocks = [&](const Box& bx) {
        const long long cols = (long long)(bx.hi[1] - bx.lo[1]) * ((bx.hi[2] - bx.lo[2]) / p->vec);
        return ((cols + kUpdThreads - 1) / kUpdThreads) * (bx.hi[0] - bx.lo[0]);
    };
    if (!sp.split) return blocks(Box{{0, 0, 0}, {p->g.nx, p->g.ny, p->g.nz}});
    long long n = blocks(sp.core);
    for (int q = 0; q < sp.n_shell; ++q) n += blocks(sp.shell[q]);
    return n;
}

template <bool HSIDE>
void batch_updates(const FdtdBatch* b, int parity, cudaStream_t st) {
    const UpdArgs* args = (HSIDE ? b->argsH : b->argsE) + parity * b->max_args;
    for (int cls = 0; cls < 4; ++cls) {
        const int n = b->class_start[cls + 1] - b->class_start[cls];
        if (!n) continue;
        const BUnit* u = b->units + b->class_start[cls];
        const int grid = std::max(1, std::min(n, b->blocks_per_sm * b->sm_count));
        switch (cls) {
            case 0: k_batch_update<HSIDE, 1, false><<<grid, kUpdBlock, 0, st>>>(u, n, args); break;
            case 1: k_batch_update<HSIDE, 1, true><<<grid, kUpdBlock, 0, st>>>(u, n, args); break;
            case 2: k_batch_update<HSIDE, 2, false><<<grid, kUpdBlock, 0, st>>>(u, n, args); break;
            default: k_batch_update<HSIDE, 2, true><<<grid, kUpdBlock, 0, st>>>(u, n, args); break;
        }
    }
}

void batch_step(const FdtdBatch* b, int parity, cudaStream_t st) {
    batch_updates<false>(b, parity, st);
    if (b->n_src_unitsE)
        k_batch_source<true><<<std::min(b->n_src_unitsE, 4 * b->sm_count), 256, 0, st>>>(b->src_unitsE, b->n_src_unitsE,
                                                                                       b->srcE, parity);
    batch_updates<true>(b, parity, st);
    if (b->n_src_unitsH)
        k_batch_source<false><<<std::min(b->n_src_unitsH, 4 * b->sm_count), 256, 0, st>>>(b->src_unitsH, b->n_src_unitsH,
                                                                                        b->srcH, parity);
    for (int dt = 0; dt < 3; ++dt) {
        const int nu = b->iface_start[dt + 1] - b->iface_start[dt];
        if (!nu) continue;
        const int2* u = b->iface_units + b->iface_start[dt];
        const int grid = std::min(nu, 4 * b->sm_count);
        if (dt == 0) k_batch_interfaces<float><<<grid, 256, 0, st>>>(u, nu, b->ifaces, parity);
        else if (dt == 1) k_batch_interfaces<__nv_bfloat16><<<grid, 256, 0, st>>>(u, nu, b->ifaces, parity);
        else k_batch_interfaces<__half><<<grid, 256, 0, st>>>(u, nu, b->ifaces, parity);
    }
    if (b->n_det_units)
        k_batch_detector<<<std::min(b->n_det_units, 8 * b->sm_count), kDetBlock, 0, st>>>(b->det_units, b->n_det_units,
                                                                                          b->dets, parity);
    if (b->n_det_red)
        k_batch_detector_finalize<<<std::min(b->n_det_red, b->sm_count), kDetBlock, 0, st>>>(b->det_red, b->n_det_red,
                                                                                            b->dets);
    k_batch_advance<<<(b->n + 127) / 128, 128, 0, st>>>(b->tps, b->n);
}

// The branch mode's streams and events (created on first use).
bool batch_branch_streams(FdtdBatch* b) {
    if (b->fork_ev) return true;
    if (cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) != cudaSuccess) return false;
    b->sim_streams.assign(b->n, nullptr);
    b->join_ev.assign(b->n, nullptr);
    for (int s = 0; s < b->n; ++s)
        if (cudaStreamCreateWithFlags(&b->sim_streams[s], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join_ev[s], cudaEventDisableTiming) != cudaSuccess)
            return false;
    return true;
}

// `steps` steps of every simulation on its own stream (its per-plan launches, TMA cores
// included), forked from and joined back to `st`.
void batch_run_branches(const FdtdBatch* b, int parity, int steps, cudaStream_t st) {
    cudaEventRecord(b->fork_ev, st);
    for (int s = 0; s < b->n; ++s) {
        const FdtdPlan* p = b->plans[s];
        const FdtdBuffers* bb = &b->bufs[s];
        cudaStream_t ss = b->sim_streams[s];
        cudaStreamWaitEvent(ss, b->fork_ev, 0);
        int par = parity;
        for (int k = 0; k < steps; ++k) {
            float* hc = p->need_hprev && par ? p->h_twin : bb->H;
            float* hn = p->need_hprev ? (par ? bb->H : p->h_twin) : bb->H;
            launch_forward_step(p, bb, hc, hn, ss);
            if (b->any_hprev) par ^= 1;
        }
        cudaEventRecord(b->join_ev[s], ss);
        cudaStreamWaitEvent(st, b->join_ev[s], 0);
    }
}

// The fused mode's tables: the batch's own device tables, read by one persistent kernel.
FdtdFusedTables fused_tables(const FdtdBatch* b) {
    FdtdFusedTables t{};
    t.units = b->units;
    t.n_units = b->n_units;
    for (int q = 0; q < 5; ++q) t.class_start[q] = b->class_start[q];
    t.argsE = b->argsE;
    t.argsH = b->argsH;
    t.max_args = b->max_args;
    t.src_unitsE = b->src_unitsE;
    t.n_src_unitsE = b->n_src_unitsE;
    t.srcE = b->srcE;
    t.src_unitsH = b->src_unitsH;
    t.n_src_unitsH = b->n_src_unitsH;
    t.srcH = b->srcH;
    t.iface_units = b->iface_units;
    for (int q = 0; q < 4; ++q) t.iface_start[q] = b->iface_start[q];
    t.ifaces = b->ifaces;
    t.det_units = b->det_units;
    t.n_det_units = b->n_det_units;
    t.dets = b->dets;
    t.det_red = b->det_red;
    t.n_det_red = b->n_det_red;
    t.tps = b->tps;
    t.n_sims = b->n;
    t.any_hprev = b->any_hprev ? 1 : 0;
    t.bar = b->fbar;
    t.err = b->ferr;
    t.spin_limit = 1ll << 26;  // >= 4 s of polling at 64 ns per poll
    return t;
}

// Runs `steps` steps from `parity` with direct launches; returns the parity after them.
int batch_run_direct(const FdtdBatch* b, int parity, int steps, cudaStream_t st) {
    if (b->mode == 2) {
        if (steps <= 0) return parity;
        FdtdFusedTables t = fused_tables(b);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &cs);
        if (cs == cudaStreamCaptureStatusNone && take_injected(g_inject_barrier)) {
            t.inject_skip = 1;
            t.spin_limit = 1 << 16;
        }
        const int rc = fdtd_fused_launch(&t, steps, parity, st);
        if (rc && !b->fused_rc) b->fused_rc = rc;
        return b->any_hprev ? parity ^ (steps & 1) : parity;
    }
    if (b->mode == 1) {
        batch_run_branches(b, parity, steps, st);
        return b->any_hprev ? parity ^ (steps & 1) : parity;
    }
    for (int s = 0; s < steps; ++s) {
        batch_step(b, parity, st);
        if (b->any_hprev) parity ^= 1;
    }
    return parity;
}

}  // namespace

extern "C" {

int fdtd_batch_create(FdtdPlan* const* plans, const FdtdBuffers* bufs, int32_t n, FdtdBatch** out) {
    if (!plans || !bufs || !out || n <= 0) return FDTD_EINVAL;
    *out = nullptr;
    FdtdBatch* b = new FdtdBatch();
    b->n = n;
    for (int s = 0; s < n; ++s) {
        FdtdPlan* p = plans[s];
        if (!p) { delete b; fprintf(stderr, "fdtd_batch_create: plan %d is NULL\n", s); return FDTD_EINVAL; }
        if (p->parts != 1) {
            delete b;
            fprintf(stderr, "fdtd_batch_create: simulation %d has complex (Bloch) fields, which batches do not run\n", s);
            return FDTD_EINVAL;
        }
        if (p->d.n_poles > 0) {
            delete b;
            fprintf(stderr, "fdtd_batch_create: simulation %d has dispersive materials, which batches do not run\n", s);
            return FDTD_EINVAL;
        }
        if (p->full_e || p->full_h) {
            delete b;
            fprintf(stderr, "fdtd_batch_create: simulation %d has full 3x3 tensor materials, which batches do not run\n", s);
            return FDTD_EINVAL;
        }
        if (int rc = check_bufs(p, &bufs[s])) {
            fprintf(stderr, "fdtd_batch_create: simulation %d: %s\n", s, p->err.c_str());
            delete b;
            return rc;
        }
        if (p->d.record_interfaces && p->d.n_slabs && !bufs[s].recording) {
            fprintf(stderr, "fdtd_batch_create: simulation %d records interfaces but has no recording buffer\n", s);
            delete b;
            return FDTD_EINVAL;
        }
        if (p->vec > 2) p->vec = 2;  // the batched kernels carry VEC 1 and 2
        b->plans.push_back(p);
        b->bufs.push_back(bufs[s]);
        b->t.push_back(0);
        b->any_hprev = b->any_hprev || p->need_hprev;
    }
    b->sm_count = plans[0]->sm_count;
    // table sizes: upper bounds over every tile choice
    long long units = 0;
    int args = 0, srcE = 0, srcH = 0, su_E = 0, su_H = 0, dets = 0, du = 0, dred = 0, nif = 0, ifu = 0;
    for (int s = 0; s < n; ++s) {
        const FdtdPlan* p = plans[s];
        units += sim_update_blocks_upper(p);
        args += 2;
        for (int q = 0; q < p->d.n_sources; ++q) {
            const DSource& so = p->src[q];
            const long long P = so.kind == FDTD_SRC_PLANE ? face_cells(p->d.sources[q]) : 1;
            const int blocks = (int)((P + 255) / 256);
            const bool onE = !(so.kind == FDTD_SRC_DIPOLE && so.magnetic);
            const bool onH = !(so.kind == FDTD_SRC_DIPOLE && !so.magnetic);
            if (onE) { ++srcE; su_E += blocks; }
            if (onH) { ++srcH; su_H += blocks; }
        }
        if (p->d.record_interfaces && p->d.n_slabs) {
            ++nif;
            ifu += (int)((p->ifc.total + 255) / 256);
        }
        for (int q = 0; q < p->d.n_detectors; ++q) {
            if (p->fused[q]) continue;
            ++dets;
            du += p->det[q].nblocks;
            if (p->det[q].reduce) ++dred;
        }
    }
    if (units > (1ll << 30)) { delete b; return FDTD_EINVAL; }
    b->max_args = args;
    b->max_units = (int)units;
    Arena ar;
    const size_t oE = ar.take(sizeof(UpdArgs) * 2 * args), oH = ar.take(sizeof(UpdArgs) * 2 * args);
    const size_t oU = ar.take(sizeof(BUnit) * units);
    const size_t oSE = ar.take(sizeof(BSrc) * std::max(1, srcE)), oSH = ar.take(sizeof(BSrc) * std::max(1, srcH));
    const size_t oSUE = ar.take(sizeof(int2) * std::max(1, su_E)), oSUH = ar.take(sizeof(int2) * std::max(1, su_H));
    const size_t oD = ar.take(sizeof(BDet) * std::max(1, dets)), oDU = ar.take(sizeof(int2) * std::max(1, du));
    const size_t oDR = ar.take(sizeof(int) * std::max(1, dred)), oT = ar.take(sizeof(int*) * n);
    const size_t oI = ar.take(sizeof(BIface) * std::max(1, nif)), oIU = ar.take(sizeof(int2) * std::max(1, ifu));
    const size_t oFB = ar.take(2 * sizeof(unsigned)), oFE = ar.take(sizeof(int));
    cudaError_t e = dev_alloc(reinterpret_cast<void**>(&b->dmem), ar.off);
    if (e != cudaSuccess) {
        fprintf(stderr, "fdtd_batch_create: cudaMalloc(%zu): %s\n", ar.off, cudaGetErrorString(e));
        delete b;
        return FDTD_ENOMEM;
    }
    b->argsE = reinterpret_cast<UpdArgs*>(b->dmem + oE);
    b->argsH = reinterpret_cast<UpdArgs*>(b->dmem + oH);
    b->units = reinterpret_cast<BUnit*>(b->dmem + oU);
    b->srcE = reinterpret_cast<BSrc*>(b->dmem + oSE);
    b->srcH = reinterpret_cast<BSrc*>(b->dmem + oSH);
    b->src_unitsE = reinterpret_cast<int2*>(b->dmem + oSUE);
    b->src_unitsH = reinterpret_cast<int2*>(b->dmem + oSUH);
    b->dets = reinterpret_cast<BDet*>(b->dmem + oD);
    b->det_units = reinterpret_cast<int2*>(b->dmem + oDU);
    b->det_red = reinterpret_cast<int*>(b->dmem + oDR);
    b->tps = reinterpret_cast<int**>(b->dmem + oT);
    b->ifaces = reinterpret_cast<BIface*>(b->dmem + oI);
    b->iface_units = reinterpret_cast<int2*>(b->dmem + oIU);
    b->fbar = reinterpret_cast<unsigned*>(b->dmem + oFB);
    b->ferr = reinterpret_cast<int*>(b->dmem + oFE);
    if (cudaMemset(b->fbar, 0, 2 * sizeof(unsigned)) != cudaSuccess || cudaMemset(b->ferr, 0, sizeof(int)) != cudaSuccess) {
        fdtd_batch_destroy(b);
        return FDTD_ECUDA;
    }
    // sources, detectors, step counters (independent of the tile choice)
    std::vector<BSrc> hsE, hsH;
    std::vector<int2> huE, huH, hdu;
    std::vector<BDet> hd;
    std::vector<int> hdr;
    std::vector<int*> htp;
    std::vector<BIface> hif;
    std::vector<int2> hifu[3];
    for (int s = 0; s < n; ++s) {
        FdtdPlan* p = plans[s];
        const FdtdBuffers& bb = bufs[s];
        float* hc[2] = {bb.H, p->need_hprev ? p->h_twin : bb.H};
        float* hn[2] = {p->need_hprev ? p->h_twin : bb.H, bb.H};
        htp.push_back(p->d_t);
        if (p->d.record_interfaces && p->d.n_slabs) {
            BIface x{};
            x.g = p->g; x.ifc = p->ifc; x.tp = p->d_t; x.n_slots = rec_rows(p->d);
            x.E = bb.E; x.H[0] = hn[0]; x.H[1] = hn[1]; x.rec = bb.recording;
            const int dt = p->d.recording_dtype >= 0 && p->d.recording_dtype <= 2 ? p->d.recording_dtype : 0;
            for (long long k = 0; k < (p->ifc.total + 255) / 256; ++k) hifu[dt].push_back(make_int2((int)hif.size(), (int)k));
            hif.push_back(x);
        }
        for (int q = 0; q < p->d.n_sources; ++q) {
            const DSource& so = p->src[q];
            const long long P = so.kind == FDTD_SRC_PLANE ? face_cells(p->d.sources[q]) : 1;
            const int blocks = (int)((P + 255) / 256);
            if (!(so.kind == FDTD_SRC_DIPOLE && so.magnetic)) {
                BSrc x{};
                x.g = p->g; x.s = so; x.tp = p->d_t; x.F[0] = x.F[1] = bb.E;
                x.mat = bb.inv_eps; x.n_mat = p->d.n_eps; x.mat_scalar = 1.f;
                for (int k = 0; k < blocks; ++k) huE.push_back(make_int2((int)hsE.size(), k));
                hsE.push_back(x);
            }
            if (!(so.kind == FDTD_SRC_DIPOLE && !so.magnetic)) {
                BSrc x{};
                x.g = p->g; x.s = so; x.tp = p->d_t; x.F[0] = hn[0]; x.F[1] = hn[1];
                x.mat = p->d.n_mu ? bb.inv_mu : nullptr; x.n_mat = p->d.n_mu ? p->d.n_mu : 1;
                x.mat_scalar = p->d.inv_mu_scalar;
                for (int k = 0; k < blocks; ++k) huH.push_back(make_int2((int)hsH.size(), k));
                hsH.push_back(x);
            }
        }
        for (int q = 0; q < p->d.n_detectors; ++q) {
            if (p->fused[q]) continue;
            BDet x{};
            x.g = p->g; x.d = p->det[q]; x.tp = p->d_t; x.state = bb.det_state[q];
            for (int par = 0; par < 2; ++par)
                x.f[par] = DetFields{bb.E, hc[par], hn[par], bb.inv_eps, p->d.n_eps, p->d.n_mu ? bb.inv_mu : nullptr,
                                     p->d.n_mu ? p->d.n_mu : 1, p->d.inv_mu_scalar};
            for (int k = 0; k < p->det[q].nblocks; ++k) hdu.push_back(make_int2((int)hd.size(), k));
            if (p->det[q].reduce) hdr.push_back((int)hd.size());
            hd.push_back(x);
        }
    }
    b->n_srcE = (int)hsE.size(); b->n_srcH = (int)hsH.size();
    b->n_src_unitsE = (int)huE.size(); b->n_src_unitsH = (int)huH.size();
    b->n_dets = (int)hd.size(); b->n_det_units = (int)hdu.size(); b->n_det_red = (int)hdr.size();
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    up(b->srcE, hsE.data(), sizeof(BSrc) * hsE.size());
    up(b->srcH, hsH.data(), sizeof(BSrc) * hsH.size());
    up(b->src_unitsE, huE.data(), sizeof(int2) * huE.size());
    up(b->src_unitsH, huH.data(), sizeof(int2) * huH.size());
    up(b->dets, hd.data(), sizeof(BDet) * hd.size());
    up(b->det_units, hdu.data(), sizeof(int2) * hdu.size());
    up(b->det_red, hdr.data(), sizeof(int) * hdr.size());
    up(b->tps, htp.data(), sizeof(int*) * htp.size());
    {
        std::vector<int2> all;
        for (int dt = 0; dt < 3; ++dt) {
            b->iface_start[dt] = (int)all.size();
            all.insert(all.end(), hifu[dt].begin(), hifu[dt].end());
        }
        b->iface_start[3] = (int)all.size();
        up(b->ifaces, hif.data(), sizeof(BIface) * hif.size());
        up(b->iface_units, all.data(), sizeof(int2) * all.size());
    }
    if (e != cudaSuccess) {
        fprintf(stderr, "fdtd_batch_create: upload: %s\n", cudaGetErrorString(e));
        cudaFree(b->dmem);
        delete b;
        return FDTD_ECUDA;
    }
    if (int rc = batch_build_updates(b)) {
        fprintf(stderr, "fdtd_batch_create: %s\n", b->err.c_str());
        cudaFree(b->dmem);
        delete b;
        return rc;
    }
    *out = b;
    return FDTD_OK;
}

void fdtd_batch_destroy(FdtdBatch* b) {
    if (!b) return;
    batch_drop_graph(b);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    for (cudaStream_t x : b->sim_streams)
        if (x) cudaStreamDestroy(x);
    for (cudaEvent_t x : b->join_ev)
        if (x) cudaEventDestroy(x);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    cudaFree(b->dmem);
    delete b;
}

const char* fdtd_batch_last_error(const FdtdBatch* b) { return b ? b->err.c_str() : "no batch"; }

int fdtd_batch_tune(FdtdBatch* b, int32_t chunk_num, int32_t chunk_den, int32_t shell_chunk, int32_t blocks_per_sm) {
    if (!b || chunk_num <= 0 || chunk_den <= 0 || shell_chunk <= 0 || blocks_per_sm <= 0 || blocks_per_sm > 64)
        return bfail(b, FDTD_EINVAL, "tile parameters must be positive (blocks_per_sm <= 64)");
    b->chunk_scale_num = chunk_num;
    b->chunk_scale_den = chunk_den;
    b->shell_chunk = shell_chunk;
    b->blocks_per_sm = blocks_per_sm;
    return batch_build_updates(b);
}

int fdtd_batch_tuning(const FdtdBatch* b, int32_t* out4) {
    if (!b || !out4) return FDTD_EINVAL;
    out4[0] = b->chunk_scale_num;
    out4[1] = b->chunk_scale_den;
    out4[2] = b->shell_chunk;
    out4[3] = b->blocks_per_sm;
    return FDTD_OK;
}

int fdtd_batch_set_mode(FdtdBatch* b, int32_t mode) {
    if (!b || mode < 0 || mode > 2) return bfail(b, FDTD_EINVAL, "mode must be 0 (persistent), 1 (branches) or 2 (fused)");
    if (mode == 1 && !batch_branch_streams(b)) return bfail(b, FDTD_ECUDA, "branch streams could not be created");
    if (mode == 2) {
        int dev = 0, coop = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
            !coop)
            return bfail(b, FDTD_EINVAL, "the fused mode needs a device with cooperative launches");
    }
    cudaDeviceSynchronize();
    b->mode = mode;
    batch_drop_graph(b);
    return FDTD_OK;
}

int32_t fdtd_batch_mode(const FdtdBatch* b) { return b ? b->mode : -1; }

int32_t fdtd_batch_launches_per_step(const FdtdBatch* b) {
    if (!b) return 0;
    if (b->mode == 2) return 1;  // one launch for all the steps of a call
    if (b->mode == 1) {
        int n = 0;
        for (const FdtdPlan* p : b->plans) n += fdtd_launches_per_step(p);
        return n;
    }
    int classes = 0;
    for (int cls = 0; cls < 4; ++cls) classes += b->class_start[cls + 1] > b->class_start[cls];
    int ifc = 0;
    for (int dt = 0; dt < 3; ++dt) ifc += b->iface_start[dt + 1] > b->iface_start[dt];
    return 2 * classes + 1 + ifc + (b->n_src_unitsE > 0) + (b->n_src_unitsH > 0) + (b->n_det_units > 0) +
           (b->n_det_red > 0);
}

}  // extern "C"

namespace {

// Times `steps` steps from *parity (updating it): under a CUDA graph captured for the purpose
// when `graph` is set (the way fdtd_batch_forward will run them; the fused mode is one launch
// either way), else as direct launches.  Returns the milliseconds, or -1 on failure.
float batch_time_steps(FdtdBatch* b, int* parity, int steps, bool graph, cudaStream_t st, cudaEvent_t e0,
                       cudaEvent_t e1) {
    float ms = -1.f;
    if (graph && b->mode != 2) {
        if (!b->cap_stream && cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess) return -1.f;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        if (cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -1.f;
        const int after = batch_run_direct(b, *parity, steps, b->cap_stream);
        const bool ok = cudaStreamEndCapture(b->cap_stream, &g) == cudaSuccess && g &&
                        cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
        if (ok) {
            cudaEventRecord(e0, st);
            if (cudaGraphLaunch(ge, st) == cudaSuccess) {
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&ms, e0, e1);
                *parity = after;
            } else {
                ms = -1.f;
            }
        }
        if (ge) cudaGraphExecDestroy(ge);
        if (g) cudaGraphDestroy(g);
        return ok ? ms : -1.f;
    }
    cudaEventRecord(e0, st);
    *parity = batch_run_direct(b, *parity, steps, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
}

// Online autotuning: times candidate tile choices on real steps (coordinate search over
// the core chunk scale, the shell chunk and the resident blocks per SM, with direct
// launches), then the best of them, the branch mode and the fused mode the way the call will
// run them (under a CUDA graph when `graph`), and keeps the fastest.  Returns the steps it
// ran and leaves the parity in *parity.
int batch_autotune(FdtdBatch* b, int budget, int* parity, bool graph, cudaStream_t st) {
    const int per = b->any_hprev ? 4 : 3;  // timed steps per candidate (even with a parity twin)
    const int warm = b->any_hprev ? 2 : 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int used = 0;
    auto fits = [&]() { return used + per + warm <= budget; };
    auto run = [&](bool as_graph) -> float {
        *parity = batch_run_direct(b, *parity, warm, st);
        const float ms = batch_time_steps(b, parity, per, as_graph, st, e0, e1);
        used += warm + per;
        return ms;
    };
    auto trial = [&](int num, int den, int shell, int bps) -> float {
        if (!fits()) return -1.f;
        b->chunk_scale_num = num; b->chunk_scale_den = den; b->shell_chunk = shell; b->blocks_per_sm = bps;
        if (batch_build_updates(b)) return -1.f;
        return run(false);
    };
    b->mode = 0;
    int best[4] = {1, 1, kShellChunk, 8};
    float best_ms = trial(best[0], best[1], best[2], best[3]);
    const int scales[][2] = {{1, 2}, {2, 1}, {4, 1}};
    for (const auto& sc : scales) {
        const float ms = trial(sc[0], sc[1], best[2], best[3]);
        if (ms > 0.f && (best_ms < 0.f || ms < best_ms)) { best_ms = ms; best[0] = sc[0]; best[1] = sc[1]; }
    }
    for (int sh : {2, 8}) {
        const float ms = trial(best[0], best[1], sh, best[3]);
        if (ms > 0.f && ms < best_ms) { best_ms = ms; best[2] = sh; }
    }
    for (int bps : {4, 16}) {
        const float ms = trial(best[0], best[1], best[2], bps);
        if (ms > 0.f && ms < best_ms) { best_ms = ms; best[3] = bps; }
    }
    b->chunk_scale_num = best[0]; b->chunk_scale_den = best[1]; b->shell_chunk = best[2]; b->blocks_per_sm = best[3];
    batch_build_updates(b);
    // the modes, each timed as the call runs it: 0 with the chosen tiles, 1 (each simulation's
    // own kernels on its own stream), 2 (one cooperative launch for all the steps)
    int dev = 0, coop = 0;
    const bool can_fuse = cudaGetDevice(&dev) == cudaSuccess &&
                          cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop;
    float mode_ms[3] = {-1.f, -1.f, -1.f};
    if (fits()) mode_ms[0] = graph ? run(true) : best_ms;
    else mode_ms[0] = best_ms;
    if (fits() && batch_branch_streams(b)) {
        b->mode = 1;
        mode_ms[1] = run(graph);
    }
    if (fits() && can_fuse) {
        b->mode = 2;
        mode_ms[2] = run(false);
        if (b->fused_rc) mode_ms[2] = -1.f;
    }
    b->mode = 0;
    for (int m = 1; m < 3; ++m)
        if (mode_ms[m] > 0.f && (mode_ms[b->mode] <= 0.f || mode_ms[m] < mode_ms[b->mode])) b->mode = m;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    batch_drop_graph(b);
    b->tuned = true;
    return used;
}

}  // namespace

extern "C" int fdtd_batch_forward(FdtdBatch* b, const int32_t* t0, int32_t n_steps, int32_t flags, void* stream) {
    NvtxRange nvtx_range("fdtd_batch_forward");
    if (!b) return FDTD_EINVAL;
    if (cudaError_t pre = cudaGetLastError(); pre != cudaSuccess)
        return bfail(b, FDTD_ECUDA, std::string("error left pending by an earlier CUDA call (before fdtd_batch_forward): ") +
                                        cudaGetErrorString(pre));
    if (n_steps < 0) return bfail(b, FDTD_EINVAL, "n_steps must be >= 0");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    for (int s = 0; s < b->n; ++s) {
        const int ts = t0 ? t0[s] : b->t[s];
        if (ts < 0 || (long long)ts + n_steps > (long long)b->plans[s]->d.n_steps_total + 1)
            return bfail(b, FDTD_EINVAL, "simulation " + std::to_string(s) + ": steps out of the range of its tables");
    }
    if (t0)
        for (int s = 0; s < b->n; ++s) {
            k_set_step<<<1, 1, 0, st>>>(b->plans[s]->d_t, t0[s]);
            b->t[s] = t0[s];
        }
    if (n_steps == 0) return FDTD_OK;
    int parity = 0, done = 0;
    if ((flags & 2) && !b->tuned) done += batch_autotune(b, n_steps / 4, &parity, (flags & 1) != 0, st);
    const bool use_graph = (flags & 1) != 0 && b->mode != 2;  // the fused mode is one launch already
    // one fixed graph length, so calls with different step counts reuse the same graph
    constexpr int G = 32;
    if (use_graph && n_steps - done >= G + 1) {
        if (parity) done += (parity = batch_run_direct(b, parity, 1, st), 1);
        if (!b->gexec || b->gsteps != G) {
            batch_drop_graph(b);
            if (!b->cap_stream) {
                cudaError_t e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
                if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, cudaGetErrorString(e));
            }
            cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("begin capture: ") + cudaGetErrorString(e));
            batch_run_direct(b, 0, G, b->cap_stream);
            e = cudaStreamEndCapture(b->cap_stream, &b->graph);
            if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("end capture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&b->gexec, b->graph, 0);
            if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("instantiate: ") + cudaGetErrorString(e));
            b->gsteps = G;
        }
        while (n_steps - done >= G) {
            cudaError_t e = cudaGraphLaunch(b->gexec, st);
            if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("graph launch: ") + cudaGetErrorString(e));
            done += G;
        }
    }
    parity = batch_run_direct(b, parity, n_steps - done, st);
    if (parity) {  // H of the parity-twin simulations sits in the twin: bring it back
        for (int s = 0; s < b->n; ++s) {
            FdtdPlan* p = b->plans[s];
            if (!p->need_hprev) continue;
            cudaError_t e = cudaMemcpyAsync(b->bufs[s].H, p->h_twin, sizeof(float) * 3 * p->g.N,
                                            cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, cudaGetErrorString(e));
        }
    }
    for (int s = 0; s < b->n; ++s) b->t[s] += n_steps;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("batch launch: ") + cudaGetErrorString(e));
    if (b->fused_rc) {
        const int rc = b->fused_rc;
        b->fused_rc = 0;
        return bfail(b, FDTD_ECUDA, std::string("fused batch launch: ") + cudaGetErrorString((cudaError_t)rc));
    }
    if (b->mode == 2) {  // read the barrier's error word (the call waits for its launch here)
        int herr = 0;
        e = cudaMemcpyAsync(&herr, b->ferr, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return bfail(b, FDTD_ECUDA, std::string("fused batch launch: ") + cudaGetErrorString(e));
        if (herr) {
            cudaMemsetAsync(b->ferr, 0, sizeof(int), st);
            cudaMemsetAsync(b->fbar, 0, 2 * sizeof(unsigned), st);
            cudaStreamSynchronize(st);
            return bfail(b, herr, "fused batch launch: a grid barrier wait ran out (the steps of this call are incomplete)");
        }
    }
    return FDTD_OK;
}
