// Host side of fdtd_adjoint (included by fdtd_plan.cu, which owns the plan type and the
// launch helpers): scratch layout, per-step launch sequence of the reversible gradient.
#pragma once

namespace {

bool det_exact_h(const DDet& d) {
    if (!d.exact) return false;
    if (d.kind == FDTD_DET_FLUX || d.kind == FDTD_DET_ENERGY) return true;
    return (d.comp_mask & 56) != 0;
}

bool det_bilinear(const DDet& d) { return d.kind == FDTD_DET_FLUX || d.kind == FDTD_DET_ENERGY; }

// Bounding box [lo - 1, hi + 1) of a detector's stencil on one axis, clipped to the grid;
// a stencil that wraps around a periodic axis takes the whole axis.
void stencil_range(int lo, int hi, int n, bool periodic, int& blo, int& bhi) {
    blo = lo - 1;
    bhi = hi + 1;
    if (periodic && (blo < 0 || bhi > n)) { blo = 0; bhi = n; return; }
    blo = std::max(blo, 0);
    bhi = std::min(bhi, n);
}

int ensure_adjoint_scratch(FdtdPlan* p) {
    if (p->amem) return FDTD_OK;
    const FdtdDesc& d = p->d;
    const long long N = p->g.N;
    const int n3[3] = {d.nx, d.ny, d.nz};
    const bool per[3] = {d.periodic[0] != 0, d.periodic[1] != 0, d.periodic[2] != 0};
    Arena ar;
    const size_t parts = (size_t)p->parts;  // complex (Bloch) fields: real parts, then imaginary parts
    const size_t o_lam = ar.take(sizeof(float) * 6 * parts * (size_t)N);
    size_t o_psi[FDTD_MAX_SLABS][4] = {};
    for (int s = 0; s < d.n_slabs; ++s) {
        const DSlab& sl = p->slab[s];
        const size_t cells = (size_t)sl.sx * sl.sy * sl.sz;
        for (int q = 0; q < 4; ++q) o_psi[s][q] = ar.take(sizeof(float) * parts * cells);
    }
    // the H-before-update box: union of the exact H-reading detectors' stencils
    DBox hp{};
    bool any = false;
    int blo[3] = {0, 0, 0}, bhi[3] = {0, 0, 0};
    for (int q = 0; q < d.n_detectors; ++q) {
        const DDet& dd = p->det[q];
        if (!det_exact_h(dd)) continue;
        for (int a = 0; a < 3; ++a) {
            int l, h;
            stencil_range(dd.lo[a], dd.hi[a], n3[a], per[a], l, h);
            blo[a] = any ? std::min(blo[a], l) : l;
            bhi[a] = any ? std::max(bhi[a], h) : h;
        }
        any = true;
    }
    size_t o_hp = 0;
    if (any) {
        for (int a = 0; a < 3; ++a) { hp.lo[a] = blo[a]; hp.n[a] = bhi[a] - blo[a]; }
        hp.M = (long long)hp.n[0] * hp.n[1] * hp.n[2];
        o_hp = ar.take(sizeof(float) * 3 * parts * (size_t)hp.M);
    }
    DBox snap[FDTD_MAX_DETECTORS] = {};
    size_t o_snap[FDTD_MAX_DETECTORS] = {};
    for (int q = 0; q < d.n_detectors; ++q) {
        const DDet& dd = p->det[q];
        if (!det_bilinear(dd)) continue;
        DBox& b = snap[q];
        for (int a = 0; a < 3; ++a) { b.lo[a] = dd.lo[a] - 1; b.n[a] = dd.hi[a] - dd.lo[a] + 2; }
        b.M = (long long)b.n[0] * b.n[1] * b.n[2];
        o_snap[q] = ar.take(sizeof(float) * 6 * parts * (size_t)b.M);
    }
    size_t o_lP[2] = {0, 0};
    if (d.n_poles > 0)
        for (int q = 0; q < 2; ++q) o_lP[q] = ar.take(sizeof(float) * 3 * (size_t)d.n_poles * (size_t)N);
    char* mem = nullptr;
    cudaError_t e = dev_alloc(reinterpret_cast<void**>(&mem), ar.off);
    if (e != cudaSuccess) return fail(p, FDTD_ENOMEM, std::string("adjoint scratch: ") + cudaGetErrorString(e));
    e = cudaMemset(mem, 0, ar.off);
    if (e != cudaSuccess) {
        cudaFree(mem);
        return cuda_fail(p, e, "adjoint scratch memset");
    }
    p->amem = mem;
    p->amem_bytes = ar.off;
    p->lam_twin[0] = reinterpret_cast<float*>(mem + o_lam);
    p->lam_twin[1] = p->lam_twin[0] + 3 * (long long)parts * N;
    for (int s = 0; s < d.n_slabs; ++s)
        for (int q = 0; q < 4; ++q) p->lpsi_twin[s][q] = reinterpret_cast<float*>(mem + o_psi[s][q]);
    p->hp = hp;
    if (any) p->hp.buf = reinterpret_cast<float*>(mem + o_hp);
    if (d.n_poles > 0)
        for (int q = 0; q < 2; ++q) p->lP_twin[q] = reinterpret_cast<float*>(mem + o_lP[q]);
    for (int q = 0; q < d.n_detectors; ++q) {
        p->snap[q] = snap[q];
        if (det_bilinear(p->det[q])) p->snap[q].buf = reinterpret_cast<float*>(mem + o_snap[q]);
    }
    return FDTD_OK;
}

// One set of cotangent buffers of the state (E, H, psi).
struct LamSet {
    float* E;
    float* H;
    float* psi[FDTD_MAX_SLABS][4];
    float* Pc = nullptr;  // polarisation cotangents (dispersive scenes, stored-state loop)
    float* Pp = nullptr;
};

// The transposed step's arguments; `part` 1 selects the imaginary parts of complex (Bloch)
// fields and of their cotangents (planar buffers).
AdjArgs make_adj(const FdtdPlan* p, const FdtdBuffers* b, const FdtdAdjointBuffers* adj, const LamSet& cur,
                 const LamSet& nxt, int part = 0) {
    AdjArgs a{};
    a.g = p->g;
    const long long fo = part ? 3 * p->g.N : 0;
    if (part) {
        a.g.pother = -3 * p->g.N;
        a.g.psign = 1.f;
    }
    a.part = part;
    a.nparts = p->parts;
    a.E = b->E + fo;
    a.H = b->H + fo;
    a.ie = b->inv_eps;
    a.n_eps = p->d.n_eps;
    a.im = p->d.n_mu ? b->inv_mu : nullptr;
    a.n_mu = p->d.n_mu ? p->d.n_mu : 1;
    a.im_scalar = p->d.inv_mu_scalar;
    a.sigE = p->d.n_sigma_E ? b->sigma_E : nullptr;
    a.n_sigE = p->d.n_sigma_E;
    a.sigH = p->d.n_sigma_H ? b->sigma_H : nullptr;
    a.n_sigH = p->d.n_sigma_H;
    a.n_slab = p->d.n_slabs;
    long long ps[FDTD_MAX_SLABS] = {};
    for (int s = 0; s < p->d.n_slabs; ++s) {
        const long long cells = (long long)p->slab[s].sx * p->slab[s].sy * p->slab[s].sz;
        ps[s] = part ? cells : 0;
        a.lpother[s] = part ? -cells : cells;
        a.slab[s] = p->slab[s];
        a.psiE1[s] = b->psi_E[s][0] + ps[s];
        a.psiE2[s] = b->psi_E[s][1] + ps[s];
        a.psiH1[s] = b->psi_H[s][0] + ps[s];
        a.psiH2[s] = b->psi_H[s][1] + ps[s];
        a.lpE[s][0] = cur.psi[s][0] + ps[s]; a.lpE[s][1] = cur.psi[s][1] + ps[s];
        a.lpH[s][0] = cur.psi[s][2] + ps[s]; a.lpH[s][1] = cur.psi[s][3] + ps[s];
        a.lpE_out[s][0] = nxt.psi[s][0] + ps[s]; a.lpE_out[s][1] = nxt.psi[s][1] + ps[s];
        a.lpH_out[s][0] = nxt.psi[s][2] + ps[s]; a.lpH_out[s][1] = nxt.psi[s][3] + ps[s];
    }
    a.lE = cur.E + fo;
    a.lH = cur.H + fo;
    a.lE_out = nxt.E + fo;
    a.lH_out = nxt.H + fo;
    a.grad_ie = adj->grad_inv_eps;
    a.grad_im = adj->grad_inv_mu;
    a.hp = p->hp;
    if (a.hp.buf) {
        a.hp.buf += part ? 3 * a.hp.M : 0;
        a.hp.other = part ? -3 * a.hp.M : 3 * a.hp.M;
    }
    for (int x = 0; x < 3; ++x) a.ax_slab[x][0] = a.ax_slab[x][1] = -1;
    for (int s = 0; s < p->d.n_slabs; ++s) {
        const int side = p->d.slabs[s].direction > 0 ? 1 : 0;
        int& slot = a.ax_slab[p->slab[s].axis][side];
        slot = slot < 0 ? s : -2;  // -2: two slabs on one face (the per-axis kernels do not apply)
    }
    for (int x = 0; x < 3; ++x)
        for (int side = 0; side < 2; ++side) {
            const int s = a.ax_slab[x][side];
            if (s < 0) continue;
            a.axs[x][side] = p->slab[s];
            for (int q = 0; q < 2; ++q) {
                a.axpE[x][side][q] = b->psi_E[s][q] + ps[s];
                a.axlp[0][x][side][q] = cur.psi[s][q] + ps[s];
                a.axlp[1][x][side][q] = cur.psi[s][2 + q] + ps[s];
                a.axlpo[0][x][side][q] = nxt.psi[s][q] + ps[s];
                a.axlpo[1][x][side][q] = nxt.psi[s][2 + q] + ps[s];
            }
        }
    return a;
}

// Whether every slab's psi array is indexable with 32-bit offsets (the fast shell kernels).
bool psi_offsets_32bit(const FdtdPlan* p) {
    for (int s = 0; s < p->d.n_slabs; ++s)
        if ((long long)p->slab[s].sx * p->slab[s].sy * p->slab[s].sz >= (1LL << 31)) return false;
    return true;
}

// Whether every face holds at most one slab (the per-axis shell kernels apply).
bool axis_table_ok(const AdjArgs& a) {
    for (int x = 0; x < 3; ++x)
        for (int side = 0; side < 2; ++side)
            if (a.ax_slab[x][side] == -2) return false;
    return true;
}

int check_adj(FdtdPlan* p, const FdtdAdjointBuffers* adj) {
    if (!adj || !adj->lam_E || !adj->lam_H) return fail(p, FDTD_EINVAL, "lam_E and lam_H buffers are required");
    for (int s = 0; s < p->d.n_slabs; ++s)
        if (!adj->lam_psi_E[s][0] || !adj->lam_psi_E[s][1] || !adj->lam_psi_H[s][0] || !adj->lam_psi_H[s][1])
            return fail(p, FDTD_EINVAL, "psi cotangent buffers required for every slab");
    if (adj->grad_inv_mu && p->d.n_mu == 0)
        return fail(p, FDTD_EINVAL, "grad_inv_mu needs an inv_mu array (n_mu 1 or 3), not a scalar inv_mu");
    if (p->full_e || p->full_h)
        return fail(p, FDTD_EINVAL, "the reversible gradient of full 3x3 tensor materials is not supported");
    return FDTD_OK;
}

enum class AdjKind { Shell, ShellGeneric, ShellFast, Core, CoreFast };

template <bool HSIDE, int VEC>
void launch_adj_kernel(const AdjArgs& a, long long blocks, AdjKind kind, cudaStream_t st) {
    const unsigned nb = (unsigned)blocks;
    if (kind == AdjKind::ShellGeneric) {
        if (HSIDE) k_adj_H<VEC, true><<<nb, kUpdBlock, 0, st>>>(a);
        else k_adj_E<VEC, true><<<nb, kUpdBlock, 0, st>>>(a);
    } else if (kind == AdjKind::ShellFast) {
        if (HSIDE) k_adj_H_shell_s<VEC><<<nb, kUpdBlock, 0, st>>>(a);
        else k_adj_E_shell_s<VEC><<<nb, kUpdBlock, 0, st>>>(a);
    } else if (kind == AdjKind::Shell) {
        if (HSIDE) k_adj_H_core<VEC, true><<<nb, kUpdBlock, 0, st>>>(a);
        else k_adj_E_core<VEC, true><<<nb, kUpdBlock, 0, st>>>(a);
    } else if (kind == AdjKind::Core) {
        if (HSIDE) k_adj_H_core<VEC, false><<<nb, kUpdBlock, 0, st>>>(a);
        else k_adj_E_core<VEC, false><<<nb, kUpdBlock, 0, st>>>(a);
    } else {
        if (HSIDE) k_adj_H_core_s<VEC><<<nb, kUpdBlock, 0, st>>>(a);
        else k_adj_E_core_s<VEC><<<nb, kUpdBlock, 0, st>>>(a);
    }
}

template <bool HSIDE>
void launch_adj_boxes(const FdtdPlan* p, AdjArgs a, const Box* boxes, const int* chunks, int n, AdjKind kind,
                      cudaStream_t st) {
    // CPML shells run one z cell per thread (more warps for their latency-bound slab loads)
    const bool shell = kind == AdjKind::Shell || kind == AdjKind::ShellFast || kind == AdjKind::ShellGeneric;
    const int vec = shell ? 1 : p->vec;
    const long long blocks = fill_boxes(p, a, boxes, chunks, n, vec);
    if (blocks <= 0) return;
    if (vec == 4) launch_adj_kernel<HSIDE, 4>(a, blocks, kind, st);
    else if (vec == 2) launch_adj_kernel<HSIDE, 2>(a, blocks, kind, st);
    else launch_adj_kernel<HSIDE, 1>(a, blocks, kind, st);
}

// Whether the fast core kernel applies: the box keeps one cell off every face (no halo),
// no conductivity, no PEC/PMC faces and, for the transposed H-step, a scalar inv_mu.
bool adj_fast_core(const FdtdPlan* p, const AdjArgs& a, const Box& core, bool hside) {
    const int n[3] = {p->g.nx, p->g.ny, p->g.nz};
    for (int x = 0; x < 3; ++x)
        if (core.lo[x] < 1 || core.hi[x] > n[x] - 1) return false;
    if (p->g.pec || p->g.pmc || a.sigE || a.sigH) return false;
    return hside ? a.im == nullptr : true;
}

// One transposed half-step: a slab-free core (the forward core shrunk by one cell next to
// every slab, since the transpose reads slab terms at the neighbours) and one launch over
// the shell boxes.
template <bool HSIDE>
void launch_adj(const FdtdPlan* p, const AdjArgs& a, cudaStream_t st) {
    const Split sp = split_boxes(p, 1);
    AdjKind shell = axis_table_ok(a) ? AdjKind::Shell : AdjKind::ShellGeneric;
    // fast shell: zero halo (no periodic axis), no conductivity, no PEC/PMC, scalar inv_mu (H)
    if (shell == AdjKind::Shell && !p->g.px && !p->g.py && !p->g.pz && !p->g.pec && !p->g.pmc && !a.sigE &&
        !a.sigH && (!HSIDE || a.im == nullptr) && psi_offsets_32bit(p))
        shell = AdjKind::ShellFast;
    if (!sp.split) {
        const Box all{{0, 0, 0}, {p->g.nx, p->g.ny, p->g.nz}};
        launch_adj_boxes<HSIDE>(p, a, &all, &p->chunk, 1, shell, st);
        return;
    }
    const AdjKind ck = adj_fast_core(p, a, sp.core, HSIDE) ? AdjKind::CoreFast : AdjKind::Core;
    launch_adj_boxes<HSIDE>(p, a, &sp.core, &p->chunk, 1, ck, st);
    int chunks[6];
    for (int q = 0; q < sp.n_shell; ++q) chunks[q] = kShellChunk;
    launch_adj_boxes<HSIDE>(p, a, sp.shell, chunks, sp.n_shell, shell, st);
}

// One step of the backward loop at t = *d_t: snapshot, reconstruction, transposed step.
void launch_adjoint_step(const FdtdPlan* p, const FdtdBuffers* b, const FdtdAdjointBuffers* adj, const LamSet& cur,
                         const LamSet& nxt, cudaStream_t st) {
    const int np = p->parts;
    const long long fo = 3 * p->g.N;
    for (int q = 0; q < p->d.n_detectors; ++q) {
        if (!adj->lam_det[q] || !p->snap[q].buf) continue;
        for (int part = 0; part < np; ++part) {
            DBox sb = p->snap[q];
            sb.buf += part * 6 * sb.M;
            Geo g = p->g;
            if (part) { g.pother = -fo; g.psign = 1.f; }
            k_adj_snap<<<(unsigned)((sb.M + 255) / 256), 256, 0, st>>>(g, sb, p->det[q].slot, p->d_t, b->E + part * fo,
                                                                        b->H + part * fo);
        }
    }
    interfaces<true>(p, b, b->H, st);
    launch_sources(p, b, false, b->H, 1, st);
    for (int part = 0; part < np; ++part) launch_H<true>(p, make_upd(p, b, false, b->E, b->H, b->H, part), st);
    // here H holds H(t) and E still E3: the detector cotangents (which read H(t) for exact
    // interpolation) complete lam H3, and the inv_mu cotangent needs E3 and H(t)
    for (int part = 0; part < np; ++part) {
        const AdjArgs a = make_adj(p, b, adj, cur, nxt, part);
        for (int q = 0; q < p->d.n_detectors; ++q) {
            if (!adj->lam_det[q]) continue;
            const DDet& dd = p->det[q];
            AdjDet x{};
            x.d = dd;
            x.lam = adj->lam_det[q];
            x.snap = p->snap[q];
            if (x.snap.buf) x.snap.buf += part * 6 * x.snap.M;
            k_adj_det<<<dd.nblocks, kDetBlock, 0, st>>>(a, x, p->d_t);
        }
        if (a.grad_im) {
            const unsigned nb = (unsigned)((p->g.N + 255) / 256);
            if (a.n_slab) k_grad_mu<true><<<nb, 256, 0, st>>>(a);
            else k_grad_mu<false><<<nb, 256, 0, st>>>(a);
        }
    }
    for (int q = 0; q < p->d.n_detectors; ++q) {
        const DDet& dd = p->det[q];
        if (adj->lam_det[q] && dd.reduce && dd.kind != FDTD_DET_PHASOR)
            k_adj_det_clear<<<1, 32, 0, st>>>(dd, adj->lam_det[q], p->d_t);
    }
    launch_sources(p, b, true, b->E, 1, st);
    for (int part = 0; part < np; ++part) launch_E<true>(p, make_upd(p, b, true, b->H, b->E, b->E, part), st);
    // the transposed H-steps of both parts (each reads lam H3 of both) before either E-step
    for (int part = 0; part < np; ++part) launch_adj<true>(p, make_adj(p, b, adj, cur, nxt, part), st);
    for (int part = 0; part < np; ++part) launch_adj<false>(p, make_adj(p, b, adj, cur, nxt, part), st);
    k_advance<<<1, 1, 0, st>>>(p->d_t, -1);
}

// One step of the backward loop over stored states (the exact checkpointing gradient): the
// transposed forward step at t with the state of step t taken from `s_t` and that of step
// t + 1 from `s_t1` -- no reconstruction.  Detector cotangents see E3 = E(t + 1) and H(t), the
// transposed steps E(t), H(t) and the stored psi of step t.
void launch_adjoint_step_stored(const FdtdPlan* p, const FdtdBuffers* s_t, const FdtdBuffers* s_t1,
                                const FdtdAdjointBuffers* adj, const LamSet& cur, const LamSet& nxt, int t,
                                cudaStream_t st) {
    k_set_step<<<1, 1, 0, st>>>(p->d_t, t);
    for (int q = 0; q < p->d.n_detectors; ++q) {
        if (!adj->lam_det[q] || !p->snap[q].buf) continue;
        const DBox& sb = p->snap[q];
        k_adj_snap<<<(unsigned)((sb.M + 255) / 256), 256, 0, st>>>(p->g, sb, p->det[q].slot, p->d_t, s_t1->E, s_t1->H);
    }
    FdtdBuffers bd = *s_t;
    bd.E = s_t1->E;
    const AdjArgs ad = make_adj(p, &bd, adj, cur, nxt, 0);
    for (int q = 0; q < p->d.n_detectors; ++q) {
        if (!adj->lam_det[q]) continue;
        AdjDet x{};
        x.d = p->det[q];
        x.lam = adj->lam_det[q];
        x.snap = p->snap[q];
        k_adj_det<<<p->det[q].nblocks, kDetBlock, 0, st>>>(ad, x, p->d_t);
    }
    for (int q = 0; q < p->d.n_detectors; ++q) {
        const DDet& dd = p->det[q];
        if (adj->lam_det[q] && dd.reduce && dd.kind != FDTD_DET_PHASOR)
            k_adj_det_clear<<<1, 32, 0, st>>>(dd, adj->lam_det[q], p->d_t);
    }
    launch_adj<true>(p, make_adj(p, s_t, adj, cur, nxt, 0), st);
    launch_adj<false>(p, make_adj(p, s_t, adj, cur, nxt, 0), st);
    if (p->d.n_poles > 0) {  // the ADE part of the E-step, after lam E(t) holds the rest
        const long long n3 = 3 * p->g.N;
        k_ade_T<<<(unsigned)((n3 + 255) / 256), 256, 0, st>>>(
            p->g, cur.E, nxt.E, cur.Pc, cur.Pp, nxt.Pc, nxt.Pp, s_t->E, s_t->disp_P_curr, s_t->disp_P_prev,
            s_t->disp_c1, s_t->disp_c2, s_t->disp_c3, p->d.n_poles, p->d.n_disp, s_t->inv_eps, p->d.n_eps,
            p->d.n_sigma_E ? s_t->sigma_E : nullptr, p->d.n_sigma_E, adj->grad_inv_eps);
    }
}

}  // namespace

extern "C" int fdtd_adjoint_stored(FdtdPlan* p, const FdtdBuffers* states, int32_t t0, int32_t n_steps,
                                   const FdtdAdjointBuffers* adj, void* stream) {
    NvtxRange nvtx_range("fdtd_adjoint_stored");
    if (!p) return FDTD_EINVAL;
    if (cudaError_t pre = cudaGetLastError(); pre != cudaSuccess)
        return cuda_fail(p, pre, "error left pending by an earlier CUDA call (before fdtd_adjoint_stored)");
    if (!states) return fail(p, FDTD_EINVAL, "states required");
    if (n_steps < 0 || t0 < 0 || (long long)t0 + n_steps > p->d.n_steps_total)
        return fail(p, FDTD_EINVAL, "stored adjoint steps out of the range covered by the plan's tables");
    for (int q = 0; q <= n_steps; ++q)
        if (int rc = check_bufs(p, &states[q])) return rc;
    if (int rc = check_adj(p, adj)) return rc;
    if (p->parts != 1) return fail(p, FDTD_EINVAL, "the stored-state gradient of complex (Bloch) fields is not supported");
    if (p->d.n_poles > 0 && (!adj->lam_P_curr || !adj->lam_P_prev))
        return fail(p, FDTD_EINVAL, "a dispersive scene needs the polarisation cotangent buffers");
    if (adj->grad_inv_mu) return fail(p, FDTD_EINVAL, "the stored-state gradient provides d/d inv_eps only");
    if (n_steps == 0) return FDTD_OK;
    if (int rc = ensure_adjoint_scratch(p)) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    LamSet user{}, twin{};
    user.E = adj->lam_E;
    user.H = adj->lam_H;
    twin.E = p->lam_twin[0];
    twin.H = p->lam_twin[1];
    for (int s = 0; s < p->d.n_slabs; ++s) {
        user.psi[s][0] = adj->lam_psi_E[s][0]; user.psi[s][1] = adj->lam_psi_E[s][1];
        user.psi[s][2] = adj->lam_psi_H[s][0]; user.psi[s][3] = adj->lam_psi_H[s][1];
        for (int q = 0; q < 4; ++q) twin.psi[s][q] = p->lpsi_twin[s][q];
    }
    user.Pc = adj->lam_P_curr;
    user.Pp = adj->lam_P_prev;
    twin.Pc = p->lP_twin[0];
    twin.Pp = p->lP_twin[1];
    const LamSet* cur = &user;
    const LamSet* nxt = &twin;
    for (int q = n_steps - 1; q >= 0; --q) {
        launch_adjoint_step_stored(p, &states[q], &states[q + 1], adj, *cur, *nxt, t0 + q, st);
        std::swap(cur, nxt);
    }
    if (cur != &user) {  // odd step count: the result sits in the twins
        const size_t fb = sizeof(float) * 3 * (size_t)p->g.N;
        cudaError_t e = cudaMemcpyAsync(user.E, cur->E, fb, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(user.H, cur->H, fb, cudaMemcpyDeviceToDevice, st);
        for (int s = 0; s < p->d.n_slabs && e == cudaSuccess; ++s) {
            const DSlab& sl = p->slab[s];
            const size_t pb = sizeof(float) * (size_t)sl.sx * sl.sy * sl.sz;
            for (int q = 0; q < 4 && e == cudaSuccess; ++q)
                e = cudaMemcpyAsync(user.psi[s][q], cur->psi[s][q], pb, cudaMemcpyDeviceToDevice, st);
        }
        if (p->d.n_poles > 0 && e == cudaSuccess) {
            const size_t pb = sizeof(float) * 3 * (size_t)p->d.n_poles * (size_t)p->g.N;
            e = cudaMemcpyAsync(user.Pc, cur->Pc, pb, cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(user.Pp, cur->Pp, pb, cudaMemcpyDeviceToDevice, st);
        }
        if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_adjoint_stored copy-back");
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_adjoint_stored launch");
    return FDTD_OK;
}

extern "C" int fdtd_adjoint(FdtdPlan* p, const FdtdBuffers* b, const FdtdAdjointBuffers* adj, int32_t t_end,
                            int32_t n_steps, void* stream) {
    NvtxRange nvtx_range("fdtd_adjoint");
    if (!p) return FDTD_EINVAL;
    if (cudaError_t pre = cudaGetLastError(); pre != cudaSuccess)
        return cuda_fail(p, pre, "error left pending by an earlier CUDA call (before fdtd_adjoint)");
    if (int rc = check_bufs(p, b)) return rc;
    if (int rc = check_adj(p, adj)) return rc;
    if (p->d.n_poles > 0) return fail(p, FDTD_EINVAL, "the reversible gradient of dispersive materials is not supported");
    if (p->parts != 1 && adj->grad_inv_mu)
        return fail(p, FDTD_EINVAL, "the inv_mu cotangent of complex (Bloch) fields is not supported (inv_eps is)");
    if (n_steps < 0 || t_end - n_steps < -1 || t_end > p->d.n_steps_total)
        return fail(p, FDTD_EINVAL, "adjoint steps out of the range covered by the plan's tables");
    if (n_steps == 0) return FDTD_OK;
    if (int rc = ensure_adjoint_scratch(p)) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    LamSet user{}, twin{};
    user.E = adj->lam_E;
    user.H = adj->lam_H;
    twin.E = p->lam_twin[0];
    twin.H = p->lam_twin[1];
    for (int s = 0; s < p->d.n_slabs; ++s) {
        user.psi[s][0] = adj->lam_psi_E[s][0]; user.psi[s][1] = adj->lam_psi_E[s][1];
        user.psi[s][2] = adj->lam_psi_H[s][0]; user.psi[s][3] = adj->lam_psi_H[s][1];
        for (int q = 0; q < 4; ++q) twin.psi[s][q] = p->lpsi_twin[s][q];
    }
    k_set_step<<<1, 1, 0, st>>>(p->d_t, t_end - 1);
    const LamSet* cur = &user;
    const LamSet* nxt = &twin;
    int done = 0;
    // an even number of steps replayed from a CUDA graph: the cotangents end where they
    // started, and every kernel reads the step from the device counter
    if (n_steps >= 16) {
        const int G = 16;
        const bool same = p->agexec && p->agsteps == G && std::memcmp(&p->agbufs, b, sizeof(FdtdBuffers)) == 0 &&
                          std::memcmp(&p->agadj, adj, sizeof(FdtdAdjointBuffers)) == 0;
        if (!same) {
            if (p->agexec) { cudaGraphExecDestroy(p->agexec); p->agexec = nullptr; }
            if (p->agraph) { cudaGraphDestroy(p->agraph); p->agraph = nullptr; }
            if (!p->cap_stream) {
                cudaError_t e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
                if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamCreate");
            }
            cudaError_t e = cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamBeginCapture");
            const LamSet* c = &user;
            const LamSet* n = &twin;
            for (int s = 0; s < G; ++s) {
                launch_adjoint_step(p, b, adj, *c, *n, p->cap_stream);
                std::swap(c, n);
            }
            e = cudaStreamEndCapture(p->cap_stream, &p->agraph);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&p->agexec, p->agraph, 0);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaGraphInstantiate");
            p->agbufs = *b;
            p->agadj = *adj;
            p->agsteps = G;
        }
        while (n_steps - done >= G) {
            cudaError_t e = cudaGraphLaunch(p->agexec, st);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaGraphLaunch");
            done += G;
        }
    }
    for (; done < n_steps; ++done) {
        launch_adjoint_step(p, b, adj, *cur, *nxt, st);
        std::swap(cur, nxt);
    }
    if (cur != &user) {  // odd step count: the result sits in the twins
        const size_t fb = sizeof(float) * 3 * (size_t)p->parts * (size_t)p->g.N;
        cudaError_t e = cudaMemcpyAsync(user.E, cur->E, fb, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(user.H, cur->H, fb, cudaMemcpyDeviceToDevice, st);
        for (int s = 0; s < p->d.n_slabs && e == cudaSuccess; ++s) {
            const DSlab& sl = p->slab[s];
            const size_t pb = sizeof(float) * (size_t)p->parts * sl.sx * sl.sy * sl.sz;
            for (int q = 0; q < 4 && e == cudaSuccess; ++q)
                e = cudaMemcpyAsync(user.psi[s][q], cur->psi[s][q], pb, cudaMemcpyDeviceToDevice, st);
        }
        if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_adjoint copy-back");
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_adjoint launch");
    return FDTD_OK;
}
