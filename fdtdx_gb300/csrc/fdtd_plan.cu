// Host side of the C ABI declared in include/fdtd_gb300.h: plan construction
// (device copies of the small per-scene tables), the per-step launch sequence,
// CUDA-graph capture of the step loop and the reverse (time-reversed) loop.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "fdtd_kernels.cuh"
#include "fdtd_aniso.cuh"
#include "fdtd_adjoint.cuh"
#include "fdtd_tma.cuh"
#include "fdtd_split.cuh"

#include <cudaTypedefs.h>
#include <nvtx3/nvToolsExt.h>

using namespace fdtd;

struct FdtdPlan {
    FdtdDesc d;  // copy of the description; host table pointers are not used after create
    Geo g;
    int n_table = 0;
    DSlab slab[FDTD_MAX_SLABS];
    DSource src[FDTD_MAX_SOURCES];
    DDet det[FDTD_MAX_DETECTORS];
    IfaceDev ifc{};
    long long iface_floats = 0;  // floats per recording slot (6 * ifc.total)
    char* dmem = nullptr;
    size_t dmem_bytes = 0;
    int* d_t = nullptr;          // device time-step counter read by every kernel
    float* h_twin = nullptr;     // second H buffer (ping-pong) when a detector needs H before the H update
    bool need_hprev = false;
    int parts = 1;               // 2 for complex (Bloch) fields: real parts, then imaginary parts
    // full 3x3 tensor half-steps (a 9-component material or conductivity on that side): two
    // passes through the curl scratch K and the field copy T (each 3 * parts * N floats)
    bool full_e = false, full_h = false;
    float* full_k = nullptr;
    float* full_t = nullptr;
    bool fused[FDTD_MAX_DETECTORS] = {};  // accumulated inside the H half-step
    int n_fused = 0;
    int chunk = 1;                        // x planes per update block
    int vec = 1;                          // z cells per thread (4, 2 or 1: nz % vec == 0)
    int shell_chunk = 4;                  // the same two for the CPML shell boxes of a split grid
    int shell_vec = 1;
    int sm_count = 1;
    // TMA-pipelined update kernels (non-periodic scenes with nz % 4 == 0)
    bool tma_ok = false;                  // the scene admits the TMA kernels
    bool use_tma = false;                 // they are selected
    int tma_tz = 32, tma_ty = 8, tma_ns = 4;
    int tma_chunk = 1;                    // x planes per block of the H kernel
    int tma_chunk_e = 1;                  // and of the E kernel
    // CPML slab cells on the TMA kernels with in-kernel slab terms (fdtd_plan_tune_shell_tma):
    // mode 1 widens the core to the whole x and y extent (the x and y slab terms in the PML
    // kernels) and leaves the two z boxes to the register-queue shell kernel; mode 2 runs the
    // whole grid in one PML launch per half-step (z terms too); mode 0 runs all six slab boxes
    // on the shell kernel; modes 3-5 run the plain TMA kernels over the whole grid and then
    // the slab cells' corrections (fdtd_split.cuh), forward and reverse steps.  Measured on the
    // 400 x 400 x 200 coupler (ms per step, one box): mode 0 0.939, mode 3 0.906, mode 4 0.894,
    // mode 5 0.884 (each half-step's faster form); on the 200 x 200 x 100 inverse-design scene
    // mode 5 lost (forward with recording 0.479 s against 0.394 s for 3000 steps: the extra
    // launches and the coarser whole-grid tiles weigh more on a small grid; the coupler at
    // 200^3: 0.313 ms mode 0 against 0.336, at 320 x 320 x 160: 0.566 against 0.532).
    // Default: mode 5 from kSplitCells cells up, else mode 0 (set at plan creation)
    int shell_tma = 0;                    // requested mode
    bool m1_ok = false, m2_ok = false;    // admissible
    // mode 3: the plain TMA kernels over the whole grid (m2_tz tile), then the CPML corrections
    // of the slab cells (fdtd_split.cuh), one launch per axis
    bool m3_ok = false;
    int m3_chunk = 1, m3_chunk_e = 1;
    // mode 4: as mode 3, with the z slabs' terms inside the TMA tiles (a column's z layer is
    // fixed along its x-march) and only the x and y slabs corrected afterwards
    bool m4_ok = false;
    int m4_chunk = 1, m4_chunk_e = 1;
    // mode 5: mode 4 for the E half-step and mode 3 for the H half-step (the H kernel with z
    // terms needs 116 registers against 80 and loses more than its corrections cost)
    int m1_chunk = 1, m1_chunk_e = 1;     // x planes per block (H, E), mode 1
    int m2_tz = 0;                        // z extent of the mode-2 tile (the core's ty rows)
    int m2_chunk = 1, m2_chunk_e = 1;
    int* d_err = nullptr;                 // kernel error word (FDTD_ETIMEOUT on a wait that ran out)
    // graph cache for the forward loop
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    FdtdBuffers gbufs{};
    int gsteps = 0;
    cudaStream_t cap_stream = nullptr;
    // graph cache for the adjoint loop (an even number of steps: the cotangents ping-pong)
    cudaGraphExec_t agexec = nullptr;
    cudaGraph_t agraph = nullptr;
    FdtdBuffers agbufs{};
    FdtdAdjointBuffers agadj{};
    int agsteps = 0;
    // reversible-gradient scratch, allocated by the first fdtd_adjoint call
    char* amem = nullptr;
    size_t amem_bytes = 0;
    float* lam_twin[2] = {nullptr, nullptr};      // cotangent twins of E and H
    float* lpsi_twin[FDTD_MAX_SLABS][4] = {};     // twins of the psi_E (1, 2) and psi_H (1, 2) cotangents
    float* lP_twin[2] = {nullptr, nullptr};       // twins of the polarisation cotangents (dispersive scenes)
    DBox hp{};                                    // H-before-update cotangents of exact detectors
    DBox snap[FDTD_MAX_DETECTORS] = {};           // (E3, H3) snapshots of bilinear detectors
    std::string err;
};

namespace {

size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// An NVTX range over one entry point (shown by Nsight tools when one is attached; a few
// nanoseconds otherwise).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Injected failures still to deliver (fdtd_debug_inject): process-wide counters.
std::atomic<int> g_inject_alloc{0};
std::atomic<int> g_inject_expiry{0};
std::atomic<int> g_inject_barrier{0};

bool take_injected(std::atomic<int>& counter) {
    int v = counter.load();
    while (v > 0)
        if (counter.compare_exchange_weak(v, v - 1)) return true;
    return false;
}

// Every device allocation of the library goes through here, so an injected allocation failure
// reaches each caller's out-of-memory path without exhausting the device.
cudaError_t dev_alloc(void** ptr, size_t bytes) {
    if (take_injected(g_inject_alloc)) {
        *ptr = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(ptr, bytes);
}

int fail(FdtdPlan* p, int code, const std::string& msg) {
    if (p) p->err = msg;
    return code;
}

int cuda_fail(FdtdPlan* p, cudaError_t e, const char* where) {
    return fail(p, FDTD_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Drops the cached CUDA graphs of the forward and adjoint loops (a tuning change alters the
// launches they hold).
void drop_graphs(FdtdPlan* p) {
    if (p->gexec) { cudaGraphExecDestroy(p->gexec); p->gexec = nullptr; }
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    p->gsteps = 0;
    if (p->agexec) { cudaGraphExecDestroy(p->agexec); p->agexec = nullptr; }
    if (p->agraph) { cudaGraphDestroy(p->agraph); p->agraph = nullptr; }
    p->agsteps = 0;
}

// Layout of the plan's single device allocation.
struct Arena {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes);
        return o;
    }
};

// Rows of the interface recording: one per step, or the time filter's stored steps.
int rec_rows(const FdtdDesc& d) { return d.rec_slots > 0 ? d.rec_slots : d.n_steps_total; }

long long face_cells(const FdtdSourceDesc& s) {
    return (long long)(s.hi[0] - s.lo[0]) * (s.hi[1] - s.lo[1]) * (s.hi[2] - s.lo[2]);
}

int popcount6(int m) {
    int c = 0;
    for (int q = 0; q < 6; ++q) c += (m >> q) & 1;
    return c;
}

int det_ncomp(const FdtdDetectorDesc& dd) {
    if (dd.kind == FDTD_DET_FIELD) return popcount6(dd.comp_mask);
    if (dd.kind == FDTD_DET_PHASOR) return dd.reduce_volume ? 2 * dd.n_freq * popcount6(dd.comp_mask) : popcount6(dd.comp_mask);
    if (dd.kind == FDTD_DET_FLUX) return dd.keep_all ? 3 : 1;
    return 1;
}

bool det_needs_h(const FdtdDetectorDesc& dd) {
    if (!dd.exact_interpolation) return false;  // non-exact detectors read H after the update only
    if (dd.kind == FDTD_DET_FLUX || dd.kind == FDTD_DET_ENERGY) return true;
    return (dd.comp_mask & 56) != 0;
}

// E-only phasor / field detectors without volume reduction are accumulated by the
// H half-step itself (all their inputs are final E values held in registers there).
bool det_fusable(const FdtdDetectorDesc& dd) {
    if (dd.kind != FDTD_DET_PHASOR && dd.kind != FDTD_DET_FIELD) return false;
    if ((dd.comp_mask & ~7) != 0 || dd.reduce_volume) return false;
    if (dd.kind == FDTD_DET_PHASOR && dd.n_freq > kMaxFuseFreq) return false;
    return true;
}

constexpr int kUpdThreads = 256;
constexpr long long kSplitCells = 12ll << 20;  // grids from this size up default to shell mode 5

int pick_vec(int nz) { return nz % 2 == 0 ? 2 : 1; }  // 4 measured slower (register pressure)

int default_chunk(int nx, int ny, int nz, int sms) {
    const int vec = pick_vec(nz);
    const long long cols = ((long long)ny * (nz / vec) + kUpdThreads - 1) / kUpdThreads;
    const long long target = (long long)sms * 24;  // ~3 waves of 8 resident 256-thread blocks per SM
    long long nchunks = (target + cols - 1) / cols;
    nchunks = std::max(1ll, std::min<long long>(nx, nchunks));
    return (int)((nx + nchunks - 1) / nchunks);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    return fn;
}

// z tile: a multiple of 4 in [8, 64] that wastes the fewest cells, the larger on ties.
// z extent of the TMA tile for a core of nz cells: the fewest staged floats per row of
// tiles, ceil(nz / tz) x (tz + 12) (the +8 z halo of the H tile and a per-tile overhead of
// about four cells), over tz in 48, 44, ..., 8.  Minimising the padding alone picks 8-cell
// tiles for a core of 184 cells (measured 1.8x slower per step than 48).
int pick_tz(int nz) {
    int best = 48;
    long long cost = 1LL << 60;
    for (int tz = 48; tz >= 8; tz -= 4) {
        const long long c = (long long)((nz + tz - 1) / tz) * (tz + 12);
        if (c < cost) { cost = c; best = tz; }
    }
    return best;
}

int align32(int x) { return (x + 31) / 32 * 32; }

// Shared-memory layout of one pipeline stage (floats): differentiated field with halo, then the
// updated field, material and conductivity tiles, each 128-byte aligned.
TmaCfg tma_cfg(int tz, int ty, int ns, bool hside, int nm, int nsig, int* err, int nd = 0) {
    TmaCfg c{};
    c.TZ = tz; c.TY = ty; c.ns = ns; c.nm = nm; c.nsig = nsig; c.nd = nd; c.err = err;
    const int fz = hside ? tz + 8 : tz + 4, fy = hside ? ty + 2 : ty + 1;
    const int nF = 3 * fy * fz, nU = 3 * ty * tz, nM = nm * ty * tz, nS = nsig * ty * tz, nD = nd * ty * 2 * tz;
    c.off_U = align32(nF);
    c.off_M = c.off_U + align32(nU);
    c.off_S = c.off_M + align32(nM);
    c.off_D = c.off_S + align32(nS);
    c.stage_floats = c.off_D + align32(nD);
    c.stage_bytes = (uint32_t)(4 * (nF + nU + nM + nS + nD));
    return c;
}

size_t tma_smem(const TmaCfg& c) { return (size_t)c.ns * c.stage_floats * 4 + (size_t)c.ns * 8; }

int validate(const FdtdDesc* d, std::string& why) {
    if (d->nx <= 0 || d->ny <= 0 || d->nz <= 0) { why = "grid dims must be positive"; return FDTD_EINVAL; }
    if ((long long)d->ny * d->nz >= (1LL << 31)) { why = "a y-z plane of 2^31 cells or more is not supported"; return FDTD_EINVAL; }
    if ((long long)d->nx * d->ny * d->nz * 3 >= (1ll << 40)) { why = "grid too large"; return FDTD_EINVAL; }
    if (d->nx > 65535) { why = "nx above 65535 is not supported"; return FDTD_EINVAL; }
    if (d->n_steps_total < 0) { why = "n_steps_total must be >= 0"; return FDTD_EINVAL; }
    auto ncomp_ok = [](int n, bool zero) { return (zero && n == 0) || n == 1 || n == 3 || n == 9; };
    if (!ncomp_ok(d->n_eps, false)) { why = "n_eps must be 1, 3 or 9"; return FDTD_EINVAL; }
    if (!ncomp_ok(d->n_mu, true)) { why = "n_mu must be 0, 1, 3 or 9"; return FDTD_EINVAL; }
    if (!ncomp_ok(d->n_sigma_E, true)) { why = "n_sigma_E must be 0, 1, 3 or 9"; return FDTD_EINVAL; }
    if (!ncomp_ok(d->n_sigma_H, true)) { why = "n_sigma_H must be 0, 1, 3 or 9"; return FDTD_EINVAL; }
    if (d->n_slabs < 0 || d->n_slabs > FDTD_MAX_SLABS) { why = "too many slabs"; return FDTD_EINVAL; }
    if (d->n_poles < 0 || (d->n_poles > 0 && d->n_disp != 1 && d->n_disp != 3)) {
        why = "dispersive poles need n_disp 1 or 3";
        return FDTD_EINVAL;
    }
    if (d->n_poles > 0 && d->bloch_axes) { why = "dispersive materials with complex (Bloch) fields are not supported"; return FDTD_EINVAL; }
    if (d->n_poles > 0 && (d->n_eps == 9 || d->n_sigma_E == 9)) {
        why = "dispersive materials with a full-tensor permittivity are not supported";
        return FDTD_EINVAL;
    }
    if (d->rec_slots < 0 || (d->rec_slots > 0 && (!d->rec_store || !d->rec_a || !d->rec_b || !d->rec_w))) {
        why = "a recorder time filter needs rec_slots > 0 and all four tables";
        return FDTD_EINVAL;
    }
    if (d->rec_slots > 0)
        for (int t = 0; t < d->n_steps_total + 2; ++t)
            if (d->rec_store[t] >= d->rec_slots || d->rec_a[t] < 0 || d->rec_a[t] >= d->rec_slots || d->rec_b[t] < 0 ||
                d->rec_b[t] >= d->rec_slots) {
                why = "recorder time-filter tables reference slots outside [0, rec_slots)";
                return FDTD_EINVAL;
            }
    if (d->n_sources < 0 || d->n_sources > FDTD_MAX_SOURCES) { why = "too many sources"; return FDTD_EINVAL; }
    if (d->n_detectors < 0 || d->n_detectors > FDTD_MAX_DETECTORS) { why = "too many detectors"; return FDTD_EINVAL; }
    const int n[3] = {d->nx, d->ny, d->nz};
    for (int s = 0; s < d->n_slabs; ++s) {
        const FdtdSlabDesc& sl = d->slabs[s];
        if (sl.axis < 0 || sl.axis > 2 || sl.thickness <= 0 || sl.thickness > n[sl.axis] || !sl.coef ||
            (sl.direction != -1 && sl.direction != 1)) {
            why = "invalid slab " + std::to_string(s);
            return FDTD_EINVAL;
        }
    }
    for (int s = 0; s < d->n_sources; ++s) {
        const FdtdSourceDesc& so = d->sources[s];
        for (int a = 0; a < 3; ++a)
            if (so.lo[a] < 0 || so.hi[a] > n[a] || so.hi[a] <= so.lo[a]) { why = "source box out of range"; return FDTD_EINVAL; }
        if (!so.phase_E || !so.phase_H || !so.teff || !so.on) { why = "source tables missing"; return FDTD_EINVAL; }
        if (so.kind == FDTD_SRC_PLANE) {
            if (so.normal_axis < 0 || so.normal_axis > 2 || so.hi[so.normal_axis] - so.lo[so.normal_axis] != 1 || !so.inc_E ||
                !so.inc_H || !so.off_E || !so.off_H || (so.e_table && so.n_e_table <= 0)) {
                why = "invalid plane source";
                return FDTD_EINVAL;
            }
        } else if (so.kind == FDTD_SRC_DIPOLE) {
            if (so.component < 0 || so.component > 2) { why = "invalid dipole component"; return FDTD_EINVAL; }
        } else {
            why = "unknown source kind";
            return FDTD_EINVAL;
        }
    }
    for (int q = 0; q < d->n_detectors; ++q) {
        const FdtdDetectorDesc& dd = d->detectors[q];
        for (int a = 0; a < 3; ++a)
            if (dd.lo[a] < 0 || dd.hi[a] > n[a] || dd.hi[a] <= dd.lo[a]) { why = "detector box out of range"; return FDTD_EINVAL; }
        if (dd.kind < 0 || dd.kind > 3 || !dd.slot) { why = "invalid detector"; return FDTD_EINVAL; }
        if ((dd.kind == FDTD_DET_FIELD || dd.kind == FDTD_DET_PHASOR) && (dd.comp_mask <= 0 || dd.comp_mask > 63)) {
            why = "invalid detector component mask";
            return FDTD_EINVAL;
        }
        if (dd.kind == FDTD_DET_PHASOR && (dd.n_freq <= 0 || dd.n_freq > FDTD_MAX_FREQS || !dd.weights)) {
            why = "invalid phasor detector";
            return FDTD_EINVAL;
        }
        if (dd.kind == FDTD_DET_FLUX && (dd.flux_axis < 0 || dd.flux_axis > 2)) { why = "invalid flux axis"; return FDTD_EINVAL; }
    }
    if (d->recording_dtype < 0 || d->recording_dtype > 2) { why = "invalid recording dtype"; return FDTD_EINVAL; }
    if (d->bloch_axes & ~7) { why = "bloch_axes holds bits beyond the three axes"; return FDTD_EINVAL; }
    for (int a = 0; a < 3; ++a)
        if ((d->bloch_axes >> a & 1) && !d->periodic[a]) { why = "a Bloch axis must be periodic"; return FDTD_EINVAL; }
    if (d->bloch_axes && d->recording_dtype != 0) {
        why = "complex (Bloch) interface recordings are stored in float32 only";
        return FDTD_EINVAL;
    }
    return FDTD_OK;
}

size_t rec_elem_bytes(int dt) { return dt == 0 ? 4 : 2; }

// The update of a half-step is split into the core box (no CPML cell; TMA or register-queue
// kernel without CPML code) and up to six shell boxes (the CPML slabs; register-queue kernel
// with the corrections), so no core warp ever waits on a scattered psi read.
struct Box {
    int lo[3], hi[3];
    bool empty() const { return hi[0] <= lo[0] || hi[1] <= lo[1] || hi[2] <= lo[2]; }
};

struct Split {
    bool split = false;  // false: one CPML launch over the whole domain
    Box core;
    int n_shell = 0;
    Box shell[6];
};

// `margin` widens every slab by that many cells on its inner side (the adjoint's core must
// not read slab cells even as neighbours).
Split split_boxes(const FdtdPlan* p, int margin = 0) {
    Split sp;
    const Geo& g = p->g;
    const int n[3] = {g.nx, g.ny, g.nz};
    int L[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for (int s = 0; s < p->d.n_slabs; ++s) {
        const int ax = p->slab[s].axis, side = p->d.slabs[s].direction > 0 ? 1 : 0;
        if (L[ax][side]) return sp;  // two slabs on one face: no split
        L[ax][side] = p->slab[s].L + margin;
    }
    const int A = g.nz % 4 == 0 ? 4 : p->vec;
    const int zlo = (L[2][0] + A - 1) / A * A, zhi = (n[2] - L[2][1]) / A * A;
    Box core{{L[0][0], L[1][0], zlo}, {n[0] - L[0][1], n[1] - L[1][1], zhi}};
    if (core.empty()) return sp;
    sp.split = true;
    sp.core = core;
    const Box cand[6] = {
        {{0, 0, 0}, {L[0][0], n[1], n[2]}},
        {{n[0] - L[0][1], 0, 0}, {n[0], n[1], n[2]}},
        {{core.lo[0], 0, 0}, {core.hi[0], L[1][0], n[2]}},
        {{core.lo[0], n[1] - L[1][1], 0}, {core.hi[0], n[1], n[2]}},
        {{core.lo[0], core.lo[1], 0}, {core.hi[0], core.hi[1], zlo}},
        {{core.lo[0], core.lo[1], zhi}, {core.hi[0], core.hi[1], n[2]}},
    };
    for (const Box& b : cand)
        if (!b.empty()) sp.shell[sp.n_shell++] = b;
    return sp;
}

// The first fused detector is staged through the H pipeline when it is a phasor whose region
// origin and z extent keep every complex tile row 16-byte aligned.
int staged_planes(const FdtdPlan* p) {
    for (int q = 0; q < p->d.n_detectors; ++q) {
        if (!p->fused[q]) continue;
        const DDet& d = p->det[q];
        if (d.kind != FDTD_DET_PHASOR || d.lo[2] % 2 || d.rz % 2 || d.nfreq * d.ncomp > 16) return 0;
        return d.nfreq * d.ncomp;
    }
    return 0;
}

// The CPML slab cells on the TMA kernels.  Mode 1: the PML kernels over the whole x and y
// extent and the core's z range (x and y terms), the z boxes on the shell kernel.  Mode 2:
// the PML kernels over the whole grid, with the z extent of their tile picked for nz.  x
// chunks of about ten (E) and six (H) waves of resident blocks, as for the core.
void configure_shell_tma(FdtdPlan* p, const Split& sp, int optin) {
    p->m1_ok = p->m2_ok = p->m3_ok = p->m4_ok = false;
    if (!sp.split || p->d.n_slabs == 0) return;
    // one slab per face (the per-axis table) and 32-bit psi offsets
    int faces[3] = {0, 0, 0};
    for (int s = 0; s < p->d.n_slabs; ++s) {
        const DSlab& sl = p->slab[s];
        if ((long long)sl.sx * sl.sy * sl.sz >= (1LL << 31)) return;
        const int side = p->d.slabs[s].direction > 0 ? 1 : 0;
        if (faces[sl.axis] >> side & 1) return;
        faces[sl.axis] |= 1 << side;
    }
    auto occ_of = [&](const void* fn, int threads, size_t sm) {
        int nb = 0;
        if ((int)sm > optin || cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, sm) != cudaSuccess)
            nb = 0;
        return nb;
    };
    auto occ_pair = [&](int tz, int ty, int& oe, int& oh) {
        const int threads = ty * tz / 2;
        const size_t smE = tma_smem(tma_cfg(tz, ty, p->tma_ns, false, p->d.n_eps, p->d.n_sigma_E, nullptr));
        const size_t smH = tma_smem(tma_cfg(tz, ty, p->tma_ns, true, p->d.n_mu, p->d.n_sigma_H, nullptr, staged_planes(p)));
        oe = std::min(occ_of((const void*)k_tma_E<false, true>, threads, smE), occ_of((const void*)k_tma_E<true, true>, threads, smE));
        oh = std::min(occ_of((const void*)k_tma_H<false, true>, threads, smH), occ_of((const void*)k_tma_H<true, true>, threads, smH));
    };
    auto chunk_for = [&](int waves, int o, long long tiles, int cx) {
        long long n = std::max(1ll, (long long)waves * o * p->sm_count / std::max(1ll, tiles));
        n = std::min<long long>(n, std::max(1, cx / 4));
        return (int)((cx + n - 1) / n);
    };
    const int nx = p->g.nx, ny = p->g.ny, nz = p->g.nz, ty = p->tma_ty;
    int oe = 0, oh = 0;
    occ_pair(p->tma_tz, ty, oe, oh);
    if (oe > 0 && oh > 0) {
        const int cz = sp.core.hi[2] - sp.core.lo[2];
        const long long tiles = (long long)((cz + p->tma_tz - 1) / p->tma_tz) * ((ny + ty - 1) / ty);
        p->m1_chunk_e = chunk_for(10, oe, tiles, nx);
        p->m1_chunk = chunk_for(6, oh, tiles, nx);
        p->m1_ok = true;
    }
    const int tz2 = p->m2_tz > 0 ? p->m2_tz : pick_tz(nz);
    if (tz2 % 4 == 0 && ty * tz2 / 2 <= 256 && ty * tz2 / 2 >= 32) {
        occ_pair(tz2, ty, oe, oh);
        if (oe > 0 && oh > 0) {
            const long long tiles = (long long)((nz + tz2 - 1) / tz2) * ((ny + ty - 1) / ty);
            p->m2_tz = tz2;
            p->m2_chunk_e = chunk_for(10, oe, tiles, nx);
            p->m2_chunk = chunk_for(6, oh, tiles, nx);
            p->m2_ok = true;
        }
        // mode 3: the plain kernels on the same whole-grid tile; real, non-dispersive fields
        // and, per axis, two disjoint slabs (the corrections of an axis run in one launch)
        bool disjoint = true;
        for (int x = 0; x < 3; ++x) {
            int lo = -1, hi = -1, llo = 0;
            for (int s = 0; s < p->d.n_slabs; ++s) {
                const DSlab& sl = p->slab[s];
                if (sl.axis != x) continue;
                if (p->d.slabs[s].direction > 0) hi = sl.lo;
                else { lo = sl.lo; llo = sl.L; }
            }
            if (lo >= 0 && hi >= 0 && lo + llo > hi) disjoint = false;
        }
        const size_t smE = tma_smem(tma_cfg(tz2, ty, p->tma_ns, false, p->d.n_eps, p->d.n_sigma_E, nullptr));
        const size_t smH = tma_smem(tma_cfg(tz2, ty, p->tma_ns, true, p->d.n_mu, p->d.n_sigma_H, nullptr, staged_planes(p)));
        const int pe = std::min(occ_of((const void*)k_tma_E<false, 0>, ty * tz2 / 2, smE),
                                occ_of((const void*)k_tma_E<true, 0>, ty * tz2 / 2, smE));
        const int ph = std::min(occ_of((const void*)k_tma_H<false, 0>, ty * tz2 / 2, smH),
                                occ_of((const void*)k_tma_H<true, 0>, ty * tz2 / 2, smH));
        const bool split_ok = disjoint && p->parts == 1 && p->d.n_poles == 0 && !p->full_e && !p->full_h;
        const long long tiles = (long long)((nz + tz2 - 1) / tz2) * ((ny + ty - 1) / ty);
        if (split_ok && pe > 0 && ph > 0) {
            p->m3_chunk_e = chunk_for(10, pe, tiles, nx);
            p->m3_chunk = chunk_for(6, ph, tiles, nx);
            p->m3_ok = p->m2_ok;
        }
        const int ze = std::min(occ_of((const void*)k_tma_E<false, 2>, ty * tz2 / 2, smE),
                                occ_of((const void*)k_tma_E<true, 2>, ty * tz2 / 2, smE));
        const int zh = std::min(occ_of((const void*)k_tma_H<false, 2>, ty * tz2 / 2, smH),
                                occ_of((const void*)k_tma_H<true, 2>, ty * tz2 / 2, smH));
        if (split_ok && ze > 0 && zh > 0) {
            p->m4_chunk_e = chunk_for(10, ze, tiles, nx);
            p->m4_chunk = chunk_for(6, zh, tiles, nx);
            p->m4_ok = p->m2_ok;
        }
    }
    cudaGetLastError();
}

// The shell mode the launches use: the requested one, lowered to what the scene admits.
int shell_tma_mode(const FdtdPlan* p) {
    if (!p->use_tma) return 0;
    if (p->shell_tma == 5 && p->m4_ok && p->m3_ok) return 5;
    if (p->shell_tma == 4 && p->m4_ok) return 4;
    if (p->shell_tma == 3 && p->m3_ok) return 3;
    if (p->shell_tma == 2 && p->m2_ok) return 2;
    if (p->shell_tma == 1 && p->m1_ok) return 1;
    return 0;
}

// Shared memory, occupancy and the x-chunk of the TMA kernels for the current tile choice.
void configure_tma(FdtdPlan* p) {
    p->use_tma = false;
    if (!p->tma_ok) return;
    const int tz = p->tma_tz, ty = p->tma_ty, ns = p->tma_ns;
    const int threads = ty * tz / 2;
    const int nmE = p->d.n_eps, nsE = p->d.n_sigma_E, nmH = p->d.n_mu, nsH = p->d.n_sigma_H;
    const size_t smE = tma_smem(tma_cfg(tz, ty, ns, false, nmE, nsE, nullptr));
    const size_t smH = tma_smem(tma_cfg(tz, ty, ns, true, nmH, nsH, nullptr, staged_planes(p)));
    int occ = 1 << 30, occ_e = 1 << 30, occ_h = 1 << 30;
    // The attribute is per kernel function and process-wide, shared by every plan: raise it
    // once to the device's opt-in maximum (a smaller plan built later must not shrink the
    // limit a larger plan's launches rely on); occupancy below uses this plan's own size.
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) optin = 0;
    auto setup = [&](const void* fn, size_t sm, int& o) {
        if ((int)sm > optin || cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
            occ = 0;
            return;
        }
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, sm) != cudaSuccess) nb = 0;
        occ = std::min(occ, nb);
        o = std::min(o, nb);
    };
    setup((const void*)k_tma_E<false>, smE, occ_e);
    setup((const void*)k_tma_E<true>, smE, occ_e);
    setup((const void*)k_tma_H<false>, smH, occ_h);
    setup((const void*)k_tma_H<true>, smH, occ_h);
    cudaGetLastError();
    if (occ <= 0 || threads > 256 || threads < 32) return;
    const Split sp = split_boxes(p);
    configure_shell_tma(p, sp, optin);
    const Box core = sp.split ? sp.core : Box{{0, 0, 0}, {p->g.nx, p->g.ny, p->g.nz}};
    const int cx = core.hi[0] - core.lo[0], cy = core.hi[1] - core.lo[1], cz = core.hi[2] - core.lo[2];
    const long long tiles = (long long)((cz + tz - 1) / tz) * ((cy + ty - 1) / ty);
    // x chunks per kernel: about ten waves of resident blocks for the E kernel and six for the
    // H kernel (measured on the 400 x 400 x 200 coupler: E 0.181 ms at 10-plane chunks against
    // 0.205 at the four-wave 43, H 0.392 ms at 26 against 0.403); fewer, longer x-marches leave
    // a long tail of lone blocks
    auto chunk_for = [&](int waves, int o) {
        long long n = std::max(1ll, (long long)waves * o * p->sm_count / tiles);
        n = std::min<long long>(n, std::max(1, cx / 4));
        return (int)((cx + n - 1) / n);
    };
    p->tma_chunk_e = chunk_for(10, occ_e);
    p->tma_chunk = chunk_for(6, occ_h);
    p->use_tma = true;
}

}  // namespace

extern "C" {

int fdtd_plan_create(const FdtdDesc* desc, FdtdPlan** out) {
    NvtxRange nvtx_range("fdtd_plan_create");
    if (!desc || !out) return FDTD_EINVAL;
    *out = nullptr;
    std::string why;
    if (int rc = validate(desc, why)) {
        // no plan exists to carry the message: print it once
        fprintf(stderr, "fdtd_plan_create: %s\n", why.c_str());
        return rc;
    }
    FdtdPlan* p = new FdtdPlan();
    p->d = *desc;
    const FdtdDesc& d = p->d;
    p->n_table = d.n_steps_total + 2;
    p->g.nx = d.nx; p->g.ny = d.ny; p->g.nz = d.nz;
    p->g.N = (long long)d.nx * d.ny * d.nz;
    p->g.px = d.periodic[0]; p->g.py = d.periodic[1]; p->g.pz = d.periodic[2];
    p->g.c = d.courant;
    p->g.eta0 = (float)(4e-7 * M_PI * 299792458.0);
    p->g.pec = d.pec_faces; p->g.pmc = d.pmc_faces;
    p->g.bloch = d.bloch_axes;
    for (int a = 0; a < 3; ++a) { p->g.bc[a] = d.bloch_cos[a]; p->g.bs[a] = d.bloch_sin[a]; }
    p->g.pother = 3 * p->g.N;
    p->g.psign = -1.f;
    p->parts = d.bloch_axes ? 2 : 1;
    p->full_e = d.n_eps == 9 || d.n_sigma_E == 9;
    p->full_h = d.n_mu == 9 || d.n_sigma_H == 9;
    const bool full = p->full_e || p->full_h;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) p->sm_count = 152;
        p->chunk = default_chunk(d.nx, d.ny, d.nz, p->sm_count);
        p->vec = pick_vec(d.nz);
        p->tma_ok = d.nz % 4 == 0 && d.nz >= 8 && !d.periodic[0] && !d.periodic[1] && !d.periodic[2] && !full && encode_fn();
        p->tma_ty = 8;
    }

    // ---- lay out the device arena
    Arena ar;
    const size_t o_t = ar.take(sizeof(int) * 4);
    std::vector<size_t> o_slab(d.n_slabs);
    for (int s = 0; s < d.n_slabs; ++s) o_slab[s] = ar.take(sizeof(float) * 6 * d.slabs[s].thickness);
    struct SrcOff { size_t incE, incH, offE, offH, phE, phH, teff, on, etab; };
    std::vector<SrcOff> o_src(d.n_sources);
    const size_t tbl = (size_t)p->n_table;
    for (int s = 0; s < d.n_sources; ++s) {
        const FdtdSourceDesc& so = d.sources[s];
        SrcOff& o = o_src[s];
        if (so.kind == FDTD_SRC_PLANE) {
            const size_t P = (size_t)face_cells(so);
            o.incE = ar.take(4 * 3 * P); o.incH = ar.take(4 * 3 * P);
            o.offE = ar.take(4 * 3 * P); o.offH = ar.take(4 * 3 * P);
            o.etab = so.e_table ? ar.take(4 * (size_t)so.n_e_table) : 0;
        }
        o.phE = ar.take(4 * tbl); o.phH = ar.take(4 * tbl); o.teff = ar.take(4 * tbl); o.on = ar.take(tbl);
    }
    struct DetOff { size_t slot, w, partial; };
    std::vector<DetOff> o_det(d.n_detectors);
    for (int q = 0; q < d.n_detectors; ++q) {
        const FdtdDetectorDesc& dd = d.detectors[q];
        DetOff& o = o_det[q];
        o.slot = ar.take(4 * tbl);
        o.w = dd.kind == FDTD_DET_PHASOR ? ar.take(8 * tbl * dd.n_freq) : 0;
        const long long R = (long long)(dd.hi[0] - dd.lo[0]) * (dd.hi[1] - dd.lo[1]) * (dd.hi[2] - dd.lo[2]);
        const long long nb = (R + kDetBlock - 1) / kDetBlock;
        const bool red = dd.reduce_volume || dd.kind == FDTD_DET_PHASOR ? dd.reduce_volume : dd.reduce_volume;
        o.partial = red ? ar.take(4 * (size_t)nb * det_ncomp(dd)) : 0;
        if (det_fusable(dd) && p->n_fused < kMaxFuse && p->parts == 1 && !full) {
            p->fused[q] = true;
            ++p->n_fused;
        } else if (det_needs_h(dd)) {
            p->need_hprev = true;
        }
    }
    size_t o_twin = 0;
    if (p->need_hprev) o_twin = ar.take(sizeof(float) * 3 * (size_t)p->parts * (size_t)p->g.N);
    size_t o_full = 0;
    if (full) o_full = ar.take(sizeof(float) * 6 * (size_t)p->parts * (size_t)p->g.N);
    size_t o_rec[4] = {0, 0, 0, 0};
    if (d.rec_slots > 0)
        for (int q = 0; q < 4; ++q) o_rec[q] = ar.take(4 * tbl);
    p->dmem_bytes = ar.off;

    cudaError_t e = dev_alloc(reinterpret_cast<void**>(&p->dmem), p->dmem_bytes);
    if (e != cudaSuccess) {
        delete p;
        fprintf(stderr, "fdtd_plan_create: cudaMalloc(%zu) failed: %s\n", ar.off, cudaGetErrorString(e));
        return FDTD_ENOMEM;
    }
    // the tables go up on a private non-blocking stream, synchronised alone: no device-wide
    // wait and no legacy-stream work, so a plan can be built on one host thread while another
    // captures a CUDA graph (the serving loop places jobs beside the running batch)
    cudaStream_t up_st = nullptr;
    e = cudaStreamCreateWithFlags(&up_st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaFree(p->dmem);
        delete p;
        fprintf(stderr, "fdtd_plan_create: cudaStreamCreate: %s\n", cudaGetErrorString(e));
        return FDTD_ECUDA;
    }
    auto up = [&](size_t off, const void* src, size_t bytes) -> cudaError_t {
        if (!bytes) return cudaSuccess;
        return cudaMemcpyAsync(p->dmem + off, src, bytes, cudaMemcpyHostToDevice, up_st);
    };
    p->d_t = reinterpret_cast<int*>(p->dmem + o_t);
    p->d_err = p->d_t + 1;
    e = cudaMemsetAsync(p->d_t, 0, sizeof(int) * 4, up_st);

    const int n3[3] = {d.nx, d.ny, d.nz};
    for (int s = 0; s < d.n_slabs && e == cudaSuccess; ++s) {
        const FdtdSlabDesc& sl = d.slabs[s];
        DSlab& ds = p->slab[s];
        ds.axis = sl.axis;
        ds.L = sl.thickness;
        ds.lo = sl.direction < 0 ? 0 : n3[sl.axis] - sl.thickness;
        ds.kappa_one = sl.kappa_is_one;
        ds.sx = sl.axis == 0 ? sl.thickness : d.nx;
        ds.sy = sl.axis == 1 ? sl.thickness : d.ny;
        ds.sz = sl.axis == 2 ? sl.thickness : d.nz;
        ds.coef = reinterpret_cast<const float*>(p->dmem + o_slab[s]);
        e = up(o_slab[s], sl.coef, sizeof(float) * 6 * sl.thickness);
        // interface layer: the slab's innermost cell layer (boundary.py:126-132)
        p->ifc.axis[s] = sl.axis;
        p->ifc.layer[s] = sl.direction < 0 ? sl.thickness - 1 : n3[sl.axis] - sl.thickness;
    }
    p->ifc.n = d.n_slabs;
    p->ifc.start[0] = 0;
    for (int s = 0; s < d.n_slabs; ++s) {
        const int a = d.slabs[s].axis;
        const long long plane = (long long)(a == 0 ? 1 : d.nx) * (a == 1 ? 1 : d.ny) * (a == 2 ? 1 : d.nz);
        p->ifc.start[s + 1] = p->ifc.start[s] + plane;
    }
    p->ifc.total = p->ifc.start[d.n_slabs];
    p->iface_floats = 6 * p->ifc.total;

    for (int s = 0; s < d.n_sources && e == cudaSuccess; ++s) {
        const FdtdSourceDesc& so = d.sources[s];
        DSource& ds = p->src[s];
        const SrcOff& o = o_src[s];
        ds.kind = so.kind; ds.comp = so.component; ds.magnetic = so.magnetic; ds.normal = so.normal_axis;
        ds.profile = so.profile;
        for (int a = 0; a < 3; ++a) { ds.lo[a] = so.lo[a]; ds.hi[a] = so.hi[a]; }
        ds.sign = so.sign; ds.coef = so.coef; ds.omega_dt = so.omega_dt; ds.ramp_inv = so.ramp_inv_steps;
        ds.t0 = so.t0_steps; ds.inv2s2 = so.inv_two_sigma2;
        ds.incE = ds.incH = ds.offE = ds.offH = nullptr;
        ds.etab = nullptr;
        ds.n_etab = 0;
        if (so.kind == FDTD_SRC_PLANE) {
            const size_t P = (size_t)face_cells(so);
            ds.incE = reinterpret_cast<const float*>(p->dmem + o.incE);
            ds.incH = reinterpret_cast<const float*>(p->dmem + o.incH);
            ds.offE = reinterpret_cast<const float*>(p->dmem + o.offE);
            ds.offH = reinterpret_cast<const float*>(p->dmem + o.offH);
            e = up(o.incE, so.inc_E, 12 * P);
            if (e == cudaSuccess) e = up(o.incH, so.inc_H, 12 * P);
            if (e == cudaSuccess) e = up(o.offE, so.off_E, 12 * P);
            if (e == cudaSuccess) e = up(o.offH, so.off_H, 12 * P);
            if (so.e_table) {
                ds.etab = reinterpret_cast<const float*>(p->dmem + o.etab);
                ds.n_etab = so.n_e_table;
                if (e == cudaSuccess) e = up(o.etab, so.e_table, 4 * (size_t)so.n_e_table);
            }
        }
        ds.phE = reinterpret_cast<const float*>(p->dmem + o.phE);
        ds.phH = reinterpret_cast<const float*>(p->dmem + o.phH);
        ds.teff = reinterpret_cast<const float*>(p->dmem + o.teff);
        ds.on = reinterpret_cast<const uint8_t*>(p->dmem + o.on);
        if (e == cudaSuccess) e = up(o.phE, so.phase_E, 4 * tbl);
        if (e == cudaSuccess) e = up(o.phH, so.phase_H, 4 * tbl);
        if (e == cudaSuccess) e = up(o.teff, so.teff, 4 * tbl);
        if (e == cudaSuccess) e = up(o.on, so.on, tbl);
    }
    for (int q = 0; q < d.n_detectors && e == cudaSuccess; ++q) {
        const FdtdDetectorDesc& dd = d.detectors[q];
        DDet& ds = p->det[q];
        const DetOff& o = o_det[q];
        ds.kind = dd.kind; ds.comp_mask = dd.comp_mask; ds.exact = dd.exact_interpolation; ds.reduce = dd.reduce_volume;
        ds.inverse = dd.inverse; ds.nfreq = dd.n_freq; ds.flux_axis = dd.flux_axis; ds.keep_all = dd.keep_all;
        ds.flux_sign = dd.flux_sign; ds.cell_weight = dd.cell_weight;
        for (int a = 0; a < 3; ++a) { ds.lo[a] = dd.lo[a]; ds.hi[a] = dd.hi[a]; }
        ds.rx = dd.hi[0] - dd.lo[0]; ds.ry = dd.hi[1] - dd.lo[1]; ds.rz = dd.hi[2] - dd.lo[2];
        ds.R = (long long)ds.rx * ds.ry * ds.rz;
        ds.nblocks = (int)((ds.R + kDetBlock - 1) / kDetBlock);
        ds.ncomp = det_ncomp(dd);
        ds.slot = reinterpret_cast<const int*>(p->dmem + o.slot);
        ds.w = dd.kind == FDTD_DET_PHASOR ? reinterpret_cast<const float2*>(p->dmem + o.w) : nullptr;
        ds.partial = o.partial ? reinterpret_cast<float*>(p->dmem + o.partial) : nullptr;
        e = up(o.slot, dd.slot, 4 * tbl);
        if (e == cudaSuccess && dd.kind == FDTD_DET_PHASOR) e = up(o.w, dd.weights, 8 * tbl * dd.n_freq);
    }
    if (p->need_hprev) p->h_twin = reinterpret_cast<float*>(p->dmem + o_twin);
    if (full) {
        p->full_k = reinterpret_cast<float*>(p->dmem + o_full);
        p->full_t = p->full_k + 3 * (size_t)p->parts * (size_t)p->g.N;
    }
    if (d.rec_slots > 0 && e == cudaSuccess) {
        e = up(o_rec[0], d.rec_store, 4 * tbl);
        if (e == cudaSuccess) e = up(o_rec[1], d.rec_a, 4 * tbl);
        if (e == cudaSuccess) e = up(o_rec[2], d.rec_b, 4 * tbl);
        if (e == cudaSuccess) e = up(o_rec[3], d.rec_w, 4 * tbl);
        p->ifc.store = reinterpret_cast<const int*>(p->dmem + o_rec[0]);
        p->ifc.ra = reinterpret_cast<const int*>(p->dmem + o_rec[1]);
        p->ifc.rb = reinterpret_cast<const int*>(p->dmem + o_rec[2]);
        p->ifc.rw = reinterpret_cast<const float*>(p->dmem + o_rec[3]);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(up_st);
    cudaStreamDestroy(up_st);
    if (e != cudaSuccess) {
        fprintf(stderr, "fdtd_plan_create: %s\n", cudaGetErrorString(e));
        cudaFree(p->dmem);
        delete p;
        return FDTD_ECUDA;
    }
    // strip the host pointers from the stored description
    for (int s = 0; s < p->d.n_slabs; ++s) p->d.slabs[s].coef = nullptr;
    for (int s = 0; s < p->d.n_sources; ++s) {
        FdtdSourceDesc& so = p->d.sources[s];
        so.inc_E = so.inc_H = so.off_E = so.off_H = so.phase_E = so.phase_H = so.teff = so.e_table = nullptr;
        so.on = nullptr;
    }
    for (int q = 0; q < p->d.n_detectors; ++q) {
        p->d.detectors[q].slot = nullptr;
        p->d.detectors[q].weights = nullptr;
    }
    p->d.rec_store = p->d.rec_a = p->d.rec_b = nullptr;
    p->d.rec_w = nullptr;
    {
        const Split sp = split_boxes(p);
        p->tma_tz = pick_tz(sp.split ? sp.core.hi[2] - sp.core.lo[2] : p->g.nz);
    }
    p->shell_tma = p->g.N >= kSplitCells ? 5 : 0;
    configure_tma(p);
    *out = p;
    return FDTD_OK;
}

void fdtd_plan_destroy(FdtdPlan* p) {
    if (!p) return;
    drop_graphs(p);
    if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
    cudaFree(p->dmem);
    cudaFree(p->amem);
    delete p;
}

const char* fdtd_last_error(const FdtdPlan* p) { return p ? p->err.c_str() : "no plan"; }

int64_t fdtd_interface_floats(const FdtdPlan* p) { return p ? p->iface_floats : 0; }

int64_t fdtd_plan_device_bytes(const FdtdPlan* p) { return p ? (int64_t)(p->dmem_bytes + p->amem_bytes) : 0; }

}  // extern "C"

// -------------------------------------------------------------------------------------
// launch helpers
// -------------------------------------------------------------------------------------
namespace {

const dim3 kUpdBlock(kUpdThreads, 1, 1);

bool make_map(CUtensorMap* m, const float* base, int ncomp, const Geo& g, int bz, int by, int bc) {
    auto fn = encode_fn();
    if (!fn || !base) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)g.nz, (cuuint64_t)g.ny, (cuuint64_t)g.nx, (cuuint64_t)ncomp};
    const cuuint64_t strides[3] = {(cuuint64_t)g.nz * 4, (cuuint64_t)g.ny * g.nz * 4, (cuuint64_t)g.N * 4};
    const cuuint32_t box[4] = {(cuuint32_t)bz, (cuuint32_t)by, 1, (cuuint32_t)bc};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launch of a TMA-pipelined half-step over the core box, or (ZP) over the z-slab shell boxes
// with their CPML terms; false when a tensor map cannot be built (the caller then uses the
// register-queue kernel).
template <bool REV, bool HSIDE, int PML = 0>
bool launch_tma(const FdtdPlan* p, const UpdArgs& a, cudaStream_t st, int tz, int chunk) {
    const Geo& g = p->g;
    const int ty = p->tma_ty;
    const int nm = a.mat ? a.n_mat : 0, nsig = a.sig ? a.n_sig : 0;
    // the staged phasor tile of the first fused detector (forward H step only)
    int nd = 0;
    CUtensorMap mD;
    std::memset(&mD, 0, sizeof(mD));
    if (HSIDE && !REV && a.n_fuse > 0 && staged_planes(p) && !((uintptr_t)a.fuse[0].state & 15)) {
        const DFuse& f = a.fuse[0];
        auto fn = encode_fn();
        const int planes = f.nfreq * f.nout;
        const cuuint64_t dims[4] = {(cuuint64_t)2 * f.rz, (cuuint64_t)f.ry, (cuuint64_t)f.rx, (cuuint64_t)planes};
        const cuuint64_t strides[3] = {(cuuint64_t)8 * f.rz, (cuuint64_t)8 * f.rz * f.ry, (cuuint64_t)8 * f.R};
        const cuuint32_t box[4] = {(cuuint32_t)(2 * tz), (cuuint32_t)ty, 1, (cuuint32_t)planes};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        if (fn && fn(&mD, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, f.state, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
            nd = planes;
    }
    TmaCfg c = tma_cfg(tz, ty, p->tma_ns, HSIDE, nm, nsig, p->d_err, nd);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (g_inject_expiry.load() > 0 && cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone)
        c.expire = take_injected(g_inject_expiry) ? 1 : 0;  // direct launches only: a graph keeps no injected node
    if (nd)
        for (int x = 0; x < 3; ++x) c.dlo[x] = a.fuse[0].lo[x];
    CUtensorMap mF, mU, mM, mS;
    std::memset(&mM, 0, sizeof(mM));
    std::memset(&mS, 0, sizeof(mS));
    const int fz = HSIDE ? tz + 8 : tz + 4, fy = HSIDE ? ty + 2 : ty + 1;
    if (!make_map(&mF, a.F, 3, g, fz, fy, 3) || !make_map(&mU, a.Uin, 3, g, tz, ty, 3)) return false;
    if (nm && !make_map(&mM, a.mat, nm, g, tz, ty, nm)) return false;
    if (nsig && !make_map(&mS, a.sig, nsig, g, tz, ty, nsig)) return false;
    UpdArgs aa = a;
    aa.chunk = chunk;
    const int bx = aa.hi[0] - aa.lo[0], by = aa.hi[1] - aa.lo[1], bz = aa.hi[2] - aa.lo[2];
    const dim3 grid((bz + tz - 1) / tz, (by + ty - 1) / ty, (bx + aa.chunk - 1) / aa.chunk);
    const dim3 block(ty * tz / 2);
    if (HSIDE) k_tma_H<REV, PML><<<grid, block, tma_smem(c), st>>>(aa, mF, mU, mM, mS, mD, c);
    else k_tma_E<REV, PML><<<grid, block, tma_smem(c), st>>>(aa, mF, mU, mM, mS, c);
    return true;
}

constexpr int kShellChunk = 4;

// Slabs that can reach a box or its one-cell rim (every slab when an axis wraps).
int box_slab_mask(const FdtdPlan* p, const Box& b) {
    if (p->g.px || p->g.py || p->g.pz) return 63;
    int m = 0;
    for (int s = 0; s < p->d.n_slabs; ++s) {
        const DSlab& sl = p->slab[s];
        if (sl.lo < b.hi[sl.axis] + 1 && sl.lo + sl.L > b.lo[sl.axis] - 1) m |= 1 << s;
    }
    return m;
}

// Fills the launch's box table; returns the number of blocks of the 1-D grid.
template <typename Args>
long long fill_boxes(const FdtdPlan* p, Args& a, const Box* boxes, const int* chunks, int n, int vec = 0) {
    if (vec <= 0) vec = p->vec;
    a.nbox = n;
    long long start = 0;
    for (int q = 0; q < n; ++q) {
        const Box& b = boxes[q];
        for (int x = 0; x < 3; ++x) { a.blo[q][x] = b.lo[x]; a.bhi[q][x] = b.hi[x]; }
        const long long cols = (long long)(b.hi[1] - b.lo[1]) * ((b.hi[2] - b.lo[2]) / vec);
        const int nbx = (int)((cols + kUpdThreads - 1) / kUpdThreads);
        const int nby = (b.hi[0] - b.lo[0] + chunks[q] - 1) / chunks[q];
        a.bchunk[q] = chunks[q];
        a.nbx[q] = nbx;
        a.bstart[q] = (int)start;
        a.bslab[q] = box_slab_mask(p, b);
        start += (long long)nbx * nby;
    }
    a.bstart[n] = (int)start;
    return start;
}

template <bool REV, bool HSIDE, bool PML>
void launch_plain_boxes(const FdtdPlan* p, UpdArgs a, const Box* boxes, const int* chunks, int n, cudaStream_t st,
                        int vec = 0) {
    if (vec <= 0) vec = p->vec;
    const long long blocks = fill_boxes(p, a, boxes, chunks, n, vec);
    if (blocks <= 0) return;
    const dim3 grid((unsigned)blocks, 1, 1);
    if (PML && a.axt && vec <= 2) {  // CPML terms through the per-axis slab table
        if (a.axt == 2) {            // no periodic axis: zero-halo neighbour loads
            if (HSIDE) {
                if (vec == 2) k_update_H<REV, 2, true, 2><<<grid, kUpdBlock, 0, st>>>(a);
                else k_update_H<REV, 1, true, 2><<<grid, kUpdBlock, 0, st>>>(a);
            } else {
                if (vec == 2) k_update_E<REV, 2, true, 2><<<grid, kUpdBlock, 0, st>>>(a);
                else k_update_E<REV, 1, true, 2><<<grid, kUpdBlock, 0, st>>>(a);
            }
        } else if (HSIDE) {
            if (vec == 2) k_update_H<REV, 2, true, 1><<<grid, kUpdBlock, 0, st>>>(a);
            else k_update_H<REV, 1, true, 1><<<grid, kUpdBlock, 0, st>>>(a);
        } else {
            if (vec == 2) k_update_E<REV, 2, true, 1><<<grid, kUpdBlock, 0, st>>>(a);
            else k_update_E<REV, 1, true, 1><<<grid, kUpdBlock, 0, st>>>(a);
        }
        return;
    }
    if (HSIDE) {
        if (vec == 4) k_update_H<REV, 4, PML><<<grid, kUpdBlock, 0, st>>>(a);
        else if (vec == 2) k_update_H<REV, 2, PML><<<grid, kUpdBlock, 0, st>>>(a);
        else k_update_H<REV, 1, PML><<<grid, kUpdBlock, 0, st>>>(a);
    } else {
        if (vec == 4) k_update_E<REV, 4, PML><<<grid, kUpdBlock, 0, st>>>(a);
        else if (vec == 2) k_update_E<REV, 2, PML><<<grid, kUpdBlock, 0, st>>>(a);
        else k_update_E<REV, 1, PML><<<grid, kUpdBlock, 0, st>>>(a);
    }
}

// The CPML corrections of a split forward half-step: one launch per axis holding slabs (both
// faces in one grid, blockIdx.y the face), in x, y, z order.
template <bool REV, bool HSIDE>
void launch_pml_corr(const UpdArgs& a, cudaStream_t st, int axes) {
    auto al8 = [](const void* q) { return q == nullptr || ((uintptr_t)q & 7) == 0; };
    auto run = [&](auto ax_tag) {
        constexpr int AX = decltype(ax_tag)::value;
        if (!(axes >> AX & 1)) return;
        const long long n0 = (long long)a.axs[AX][0].sx * a.axs[AX][0].sy * a.axs[AX][0].sz * (a.axs[AX][0].L > 0);
        const long long n1 = (long long)a.axs[AX][1].sx * a.axs[AX][1].sy * a.axs[AX][1].sz * (a.axs[AX][1].L > 0);
        const long long n = std::max(n0, n1);
        if (n <= 0) return;
        if (AX == 2) {  // two cells per thread where the rows, origins and arrays allow float2 access
            bool pairs = a.g.nz % 2 == 0 && al8(a.F) && al8(a.Uout) && al8(a.mat) && al8(a.sig);
            for (int side = 0; side < 2; ++side) {
                const DSlab& sl = a.axs[2][side];
                if (sl.L == 0) continue;
                pairs = pairs && sl.L % 2 == 0 && sl.lo % 2 == 0 && al8(a.axp[2][side][0]) && al8(a.axp[2][side][1]);
            }
            if (pairs) {
                k_pml_corr_z2<REV, HSIDE><<<dim3((unsigned)((n / 2 + 255) / 256), 2), 256, 0, st>>>(a);
                return;
            }
        }
        k_pml_corr<REV, HSIDE, AX><<<dim3((unsigned)((n + 255) / 256), 2), 256, 0, st>>>(a);
    };
    run(std::integral_constant<int, 0>{});
    run(std::integral_constant<int, 1>{});
    run(std::integral_constant<int, 2>{});
}

// `mid` (optional) is recorded between the core and the shell launches (profiling).
template <bool REV, bool HSIDE>
void launch_half(const FdtdPlan* p, const UpdArgs& a, cudaStream_t st, cudaEvent_t mid = nullptr) {
    const Split sp = split_boxes(p);
    if (!sp.split) {
        const Box all{{0, 0, 0}, {p->g.nx, p->g.ny, p->g.nz}};
        if (mid) cudaEventRecord(mid, st);
        launch_plain_boxes<REV, HSIDE, true>(p, a, &all, &p->chunk, 1, st);
        return;
    }
    const int mode0 = a.axt == 2 ? shell_tma_mode(p) : 0;
    const int mode = mode0 == 5 ? (HSIDE ? 3 : 4) : mode0;
    if (mode == 3 || mode == 4) {
        // the plain update of every cell in one TMA launch (mode 4: with the z slabs' terms in
        // the tiles), then the other slab cells' CPML terms
        UpdArgs ax = a;
        for (int x = 0; x < 3; ++x) { ax.lo[x] = 0; ax.hi[x] = x == 0 ? p->g.nx : x == 1 ? p->g.ny : p->g.nz; }
        const bool ok = mode == 4 ? launch_tma<REV, HSIDE, 2>(p, ax, st, p->m2_tz, HSIDE ? p->m4_chunk : p->m4_chunk_e)
                                  : launch_tma<REV, HSIDE, 0>(p, ax, st, p->m2_tz, HSIDE ? p->m3_chunk : p->m3_chunk_e);
        if (ok) {
            if (mid) cudaEventRecord(mid, st);
            launch_pml_corr<REV, HSIDE>(a, st, mode == 4 ? 3 : 7);
            return;
        }
    }
    if (mode == 2) {
        // the whole grid in one launch of the PML kernels (every slab term in the tiles)
        UpdArgs ax = a;
        for (int x = 0; x < 3; ++x) { ax.lo[x] = 0; ax.hi[x] = x == 0 ? p->g.nx : x == 1 ? p->g.ny : p->g.nz; }
        if (mid) cudaEventRecord(mid, st);
        if (launch_tma<REV, HSIDE, true>(p, ax, st, p->m2_tz, HSIDE ? p->m2_chunk : p->m2_chunk_e)) return;
    }
    if (mode == 1) {
        // the core widened over the x and y slabs (their terms in the PML kernels), then the two
        // z boxes (over the whole x and y extent) on the shell kernel
        UpdArgs ax = a;
        ax.lo[0] = 0; ax.lo[1] = 0; ax.lo[2] = sp.core.lo[2];
        ax.hi[0] = p->g.nx; ax.hi[1] = p->g.ny; ax.hi[2] = sp.core.hi[2];
        if (launch_tma<REV, HSIDE, true>(p, ax, st, p->tma_tz, HSIDE ? p->m1_chunk : p->m1_chunk_e)) {
            if (mid) cudaEventRecord(mid, st);
            Box zb[2];
            int nzb = 0;
            if (sp.core.lo[2] > 0) zb[nzb++] = Box{{0, 0, 0}, {p->g.nx, p->g.ny, sp.core.lo[2]}};
            if (sp.core.hi[2] < p->g.nz) zb[nzb++] = Box{{0, 0, sp.core.hi[2]}, {p->g.nx, p->g.ny, p->g.nz}};
            const int zc[2] = {p->shell_chunk, p->shell_chunk};
            if (nzb) launch_plain_boxes<REV, HSIDE, true>(p, a, zb, zc, nzb, st, p->shell_vec);
            return;
        }
    }
    UpdArgs ac = a;
    for (int x = 0; x < 3; ++x) { ac.lo[x] = sp.core.lo[x]; ac.hi[x] = sp.core.hi[x]; }
    if (!(p->use_tma && launch_tma<REV, HSIDE>(p, ac, st, p->tma_tz, HSIDE ? p->tma_chunk : p->tma_chunk_e)))
        launch_plain_boxes<REV, HSIDE, false>(p, a, &sp.core, &p->chunk, 1, st);
    if (mid) cudaEventRecord(mid, st);
    int chunks[6];
    for (int q = 0; q < sp.n_shell; ++q) chunks[q] = p->shell_chunk;
    // the shells run one z cell per thread by default: fewer registers per thread, more
    // warps in flight for their latency-bound CPML and phasor loads (measured 14% (H) and
    // 24% (E) faster than two)
    launch_plain_boxes<REV, HSIDE, true>(p, a, sp.shell, chunks, sp.n_shell, st, p->shell_vec);
}

int half_step_launches(const FdtdPlan* p, bool hside) {
    const Split sp = split_boxes(p);
    if (!sp.split) return 1;
    const int mode0 = shell_tma_mode(p);
    const int mode = mode0 == 5 ? (hside ? 3 : 4) : mode0;
    if (mode == 3 || mode == 4) {  // the plain launch, one correction launch per slab axis
        int axes[3] = {0, 0, 0};
        for (int s = 0; s < p->d.n_slabs; ++s) axes[p->slab[s].axis] = 1;
        return 1 + axes[0] + axes[1] + (mode == 3 ? axes[2] : 0);
    }
    if (mode == 2) return 1;
    if (mode == 1) return 1 + ((sp.core.lo[2] > 0 || sp.core.hi[2] < p->g.nz) ? 1 : 0);
    return 1 + (sp.n_shell > 0);
}

template <bool REV>
void launch_E(const FdtdPlan* p, const UpdArgs& a, cudaStream_t st) { launch_half<REV, false>(p, a, st); }

template <bool REV>
void launch_H(const FdtdPlan* p, const UpdArgs& a, cudaStream_t st) { launch_half<REV, true>(p, a, st); }

UpdArgs make_upd(const FdtdPlan* p, const FdtdBuffers* b, bool eside, const float* F, const float* Uin, float* Uout,
                 int part = 0);
UpdArgs make_upd_fwd_H(const FdtdPlan* p, const FdtdBuffers* b, const float* Hin, float* Hout);

// A full 3x3 tensor half-step over every part: the curl pass of each part, then the tensor
// pass of each part (a wrapped neighbour of one part mixes in the other part's K and T).
template <bool REV, bool HSIDE>
void launch_full(const FdtdPlan* p, const FdtdBuffers* b, const float* F, const float* Uin, float* Uout, cudaStream_t st) {
    const long long N3 = 3 * p->g.N;
    const unsigned blocks = (unsigned)((p->g.N + 255) / 256);
    const bool inplace = Uin == Uout;
    for (int part = 0; part < p->parts; ++part)
        k_full_curl<REV, HSIDE><<<blocks, 256, 0, st>>>(make_upd(p, b, !HSIDE, F, Uin, Uout, part), p->full_k + part * N3,
                                                        inplace ? p->full_t + part * N3 : nullptr);
    for (int part = 0; part < p->parts; ++part) {
        const UpdArgs a = make_upd(p, b, !HSIDE, F, Uin, Uout, part);
        k_full_apply<REV, HSIDE><<<blocks, 256, 0, st>>>(a, p->full_k + part * N3, inplace ? p->full_t + part * N3 : a.Uin);
    }
}

// One half-step of every part: the tensor passes on a full-tensor side, else the core / shell
// launches part by part (the forward H step of real fields with its fused detectors).
template <bool REV, bool HSIDE>
void launch_side(const FdtdPlan* p, const FdtdBuffers* b, const float* F, const float* Uin, float* Uout, cudaStream_t st) {
    if (HSIDE ? p->full_h : p->full_e) {
        launch_full<REV, HSIDE>(p, b, F, Uin, Uout, st);
        return;
    }
    if (HSIDE && !REV && p->parts == 1) {
        launch_half<false, true>(p, make_upd_fwd_H(p, b, Uin, Uout), st);
        return;
    }
    for (int part = 0; part < p->parts; ++part) launch_half<REV, HSIDE>(p, make_upd(p, b, !HSIDE, F, Uin, Uout, part), st);
}

// Launches of one half-step of every part.
int side_launches(const FdtdPlan* p, bool hside) {
    if (hside ? p->full_h : p->full_e) return 2 * p->parts;
    return p->parts * half_step_launches(p, hside);
}

// The arguments of one half-step; `part` 1 selects the imaginary parts of complex (Bloch)
// fields (planar buffers: the real parts, then the imaginary parts).
UpdArgs make_upd(const FdtdPlan* p, const FdtdBuffers* b, bool eside, const float* F, const float* Uin, float* Uout,
                 int part) {
    UpdArgs a{};
    a.g = p->g;
    const long long po = part ? 3 * p->g.N : 0;
    a.F = F + po;
    a.Uin = Uin + po;
    a.Uout = Uout + po;
    if (part) {
        a.g.pother = -3 * p->g.N;
        a.g.psign = 1.f;
    }
    if (eside) {
        a.mat = b->inv_eps; a.n_mat = p->d.n_eps; a.mat_scalar = 1.f;
        a.sig = p->d.n_sigma_E ? b->sigma_E : nullptr; a.n_sig = p->d.n_sigma_E;
    } else {
        a.mat = p->d.n_mu ? b->inv_mu : nullptr; a.n_mat = p->d.n_mu ? p->d.n_mu : 1; a.mat_scalar = p->d.inv_mu_scalar;
        a.sig = p->d.n_sigma_H ? b->sigma_H : nullptr; a.n_sig = p->d.n_sigma_H;
    }
    a.n_slab = p->d.n_slabs;
    for (int s = 0; s < p->d.n_slabs; ++s) {
        a.slab[s] = p->slab[s];
        const long long ps = part ? (long long)p->slab[s].sx * p->slab[s].sy * p->slab[s].sz : 0;
        a.psi1[s] = (eside ? b->psi_E[s][0] : b->psi_H[s][0]) + ps;
        a.psi2[s] = (eside ? b->psi_E[s][1] : b->psi_H[s][1]) + ps;
    }
    // per-axis slab table: one slab per face, the two slabs of an axis disjoint
    a.axt = 1;
    for (int s = 0; s < p->d.n_slabs && a.axt; ++s) {
        const DSlab& sl = p->slab[s];
        const int side = p->d.slabs[s].direction > 0 ? 1 : 0;
        if (a.axs[sl.axis][side].L) { a.axt = 0; break; }
        a.axs[sl.axis][side] = sl;
        a.axp[sl.axis][side][0] = a.psi1[s];
        a.axp[sl.axis][side][1] = a.psi2[s];
        if ((long long)sl.sx * sl.sy * sl.sz >= (1LL << 31)) a.axt = 0;  // 32-bit psi offsets
    }
    for (int x = 0; x < 3 && a.axt; ++x) {
        const DSlab& lo = a.axs[x][0];
        const DSlab& hi = a.axs[x][1];
        if (lo.L && hi.L && lo.lo < hi.lo + hi.L && hi.lo < lo.lo + lo.L) a.axt = 0;
    }
    if (a.axt && !p->g.px && !p->g.py && !p->g.pz) a.axt = 2;  // and a zero halo on every axis
    a.chunk = p->chunk;
    a.tp = p->d_t;
    a.n_fuse = 0;
    a.lo[0] = a.lo[1] = a.lo[2] = 0;
    a.hi[0] = p->g.nx; a.hi[1] = p->g.ny; a.hi[2] = p->g.nz;
    return a;
}

// The forward H step also accumulates the fused detectors.
UpdArgs make_upd_fwd_H(const FdtdPlan* p, const FdtdBuffers* b, const float* Hin, float* Hout) {
    UpdArgs a = make_upd(p, b, false, b->E, Hin, Hout, 0);
    for (int q = 0; q < p->d.n_detectors; ++q) {
        if (!p->fused[q]) continue;
        const DDet& dd = p->det[q];
        DFuse& f = a.fuse[a.n_fuse++];
        f.kind = dd.kind; f.exact = dd.exact; f.mask = dd.comp_mask; f.nout = dd.ncomp; f.nfreq = dd.nfreq;
        f.inverse = dd.inverse;
        for (int x = 0; x < 3; ++x) { f.lo[x] = dd.lo[x]; f.hi[x] = dd.hi[x]; }
        f.rx = dd.rx; f.ry = dd.ry; f.rz = dd.rz; f.R = dd.R;
        f.slot = dd.slot; f.w = dd.w; f.state = b->det_state[q];
    }
    return a;
}

void launch_sources(const FdtdPlan* p, const FdtdBuffers* b, bool eside, float* F, int inverse, cudaStream_t st) {
    for (int s = 0; s < p->d.n_sources; ++s) {
        const DSource& so = p->src[s];
        if (so.kind == FDTD_SRC_DIPOLE && (bool)so.magnetic == eside) continue;
        const long long P = so.kind == FDTD_SRC_PLANE
                                ? (long long)(so.hi[0] - so.lo[0]) * (so.hi[1] - so.lo[1]) * (so.hi[2] - so.lo[2])
                                : 1;
        const int blocks = (int)((P + 255) / 256);
        if (eside)
            k_source<true><<<blocks, 256, 0, st>>>(p->g, so, p->d_t, F, b->inv_eps, p->d.n_eps, 1.f, inverse);
        else
            k_source<false><<<blocks, 256, 0, st>>>(p->g, so, p->d_t, F, p->d.n_mu ? b->inv_mu : nullptr,
                                                    p->d.n_mu ? p->d.n_mu : 1, p->d.inv_mu_scalar, inverse);
    }
}

int sources_launched(const FdtdPlan* p, bool eside) {
    int n = 0;
    for (int s = 0; s < p->d.n_sources; ++s) {
        const DSource& so = p->src[s];
        if (so.kind == FDTD_SRC_DIPOLE && (bool)so.magnetic == eside) continue;
        ++n;
    }
    return n;
}

template <typename T, bool RESTORE>
void launch_ifaces(const FdtdPlan* p, const FdtdBuffers* b, float* H, cudaStream_t st) {
    const int blocks = (int)((p->ifc.total + 255) / 256);
    // complex fields: the imaginary parts' planes go to a second recording after the first
    const long long fo = 3 * p->g.N, ro = (long long)rec_rows(p->d) * 6 * p->ifc.total;
    for (int part = 0; part < p->parts; ++part)
        k_interfaces<T, RESTORE><<<blocks, 256, 0, st>>>(p->g, p->ifc, p->d_t, rec_rows(p->d), b->E + part * fo,
                                                         H + part * fo, reinterpret_cast<T*>(b->recording) + part * ro);
}

template <bool RESTORE>
void interfaces(const FdtdPlan* p, const FdtdBuffers* b, float* H, cudaStream_t st) {
    if (!p->d.n_slabs || !b->recording) return;
    if (p->d.recording_dtype == 0) launch_ifaces<float, RESTORE>(p, b, H, st);
    else if (p->d.recording_dtype == 1) launch_ifaces<__nv_bfloat16, RESTORE>(p, b, H, st);
    else launch_ifaces<__half, RESTORE>(p, b, H, st);
}

// The detector inputs: the fields (with the imaginary parts' offset when they are complex) and
// the materials.
DetFields det_fields(const FdtdPlan* p, const FdtdBuffers* b, const float* Hprev, const float* H) {
    DetFields f{b->E, Hprev, H, b->inv_eps, p->d.n_eps, p->d.n_mu ? b->inv_mu : nullptr, p->d.n_mu ? p->d.n_mu : 1,
                p->d.inv_mu_scalar};
    f.im = p->parts == 2 ? 3 * p->g.N : 0;
    return f;
}

// One forward step (fdtdx/fdtd/forward.py:83-156): update_E, E sources (+PEC inside the
// update), update_H, H sources (+PMC), interface recording, detectors, advance t.
void launch_forward_step(const FdtdPlan* p, const FdtdBuffers* b, float* Hcur, float* Hnext, cudaStream_t st) {
    if (p->d.n_poles > 0) {
        const long long n = 3 * p->g.N;
        k_ade<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p->g, b->E, b->disp_P_curr, b->disp_P_prev, b->disp_c1, b->disp_c2,
                                                           b->disp_c3, p->d.n_poles, p->d.n_disp, b->inv_eps, p->d.n_eps,
                                                           p->d.n_sigma_E ? b->sigma_E : nullptr, p->d.n_sigma_E);
    }
    launch_side<false, false>(p, b, Hcur, b->E, b->E, st);
    launch_sources(p, b, true, b->E, 0, st);  // sources are real: they drive the real parts
    launch_side<false, true>(p, b, b->E, Hcur, Hnext, st);
    launch_sources(p, b, false, Hnext, 0, st);
    if (p->d.record_interfaces) interfaces<false>(p, b, Hnext, st);
    const DetFields f = det_fields(p, b, Hcur, Hnext);
    for (int q = 0; q < p->d.n_detectors; ++q) {
        if (p->fused[q]) continue;
        const DDet& dd = p->det[q];
        k_detector<<<dd.nblocks, kDetBlock, 0, st>>>(p->g, dd, p->d_t, f, b->det_state[q]);
        if (dd.reduce) k_detector_finalize<<<1, kDetBlock, 0, st>>>(dd, p->d_t, b->det_state[q]);
    }
    k_advance<<<1, 1, 0, st>>>(p->d_t, 1);
}

int check_bufs(FdtdPlan* p, const FdtdBuffers* b) {
    if (!b || !b->E || !b->H || !b->inv_eps) return fail(p, FDTD_EINVAL, "E, H and inv_eps buffers are required");
    if (p->d.n_mu && !b->inv_mu) return fail(p, FDTD_EINVAL, "inv_mu buffer required");
    if (p->d.n_sigma_E && !b->sigma_E) return fail(p, FDTD_EINVAL, "sigma_E buffer required");
    if (p->d.n_sigma_H && !b->sigma_H) return fail(p, FDTD_EINVAL, "sigma_H buffer required");
    for (int s = 0; s < p->d.n_slabs; ++s)
        if (!b->psi_E[s][0] || !b->psi_E[s][1] || !b->psi_H[s][0] || !b->psi_H[s][1])
            return fail(p, FDTD_EINVAL, "psi buffers required for every slab");
    for (int q = 0; q < p->d.n_detectors; ++q)
        if (!b->det_state[q]) return fail(p, FDTD_EINVAL, "detector state buffer missing");
    if (p->d.n_poles > 0 && (!b->disp_P_curr || !b->disp_P_prev || !b->disp_c1 || !b->disp_c2 || !b->disp_c3))
        return fail(p, FDTD_EINVAL, "a dispersive scene needs the polarisation and coefficient buffers");
    // the update kernels read and write `vec` consecutive floats at once
    const uintptr_t mask = (uintptr_t)(4 * p->vec - 1);
    const void* vecbufs[] = {b->E, b->H, b->inv_eps, b->inv_mu, b->sigma_E, b->sigma_H};
    for (const void* q : vecbufs)
        if (q && ((uintptr_t)q & mask)) return fail(p, FDTD_EINVAL, "field and material buffers must be 16-byte aligned");
    return FDTD_OK;
}

}  // namespace

extern "C" {

int32_t fdtd_launches_per_step(const FdtdPlan* p) {
    if (!p) return 0;
    int n = side_launches(p, false) + side_launches(p, true) + sources_launched(p, true) + sources_launched(p, false) + 1;
    if (p->d.n_poles > 0) ++n;
    if (p->d.record_interfaces && p->d.n_slabs) n += p->parts;
    for (int q = 0; q < p->d.n_detectors; ++q)
        if (!p->fused[q]) n += p->det[q].reduce ? 2 : 1;
    return n;
}

int fdtd_forward(FdtdPlan* p, const FdtdBuffers* b, int32_t t0, int32_t n_steps, int32_t flags, void* stream) {
    NvtxRange nvtx_range("fdtd_forward");
    if (!p) return FDTD_EINVAL;
    if (cudaError_t pre = cudaGetLastError(); pre != cudaSuccess)
        return cuda_fail(p, pre, "error left pending by an earlier CUDA call (before fdtd_forward)");
    if (int rc = check_bufs(p, b)) return rc;
    if (n_steps < 0 || t0 < 0 || (long long)t0 + n_steps > (long long)p->d.n_steps_total + 1)
        return fail(p, FDTD_EINVAL, "time steps out of the range covered by the plan's tables");
    if (p->d.record_interfaces && p->d.n_slabs && !b->recording) return fail(p, FDTD_EINVAL, "recording buffer required");
    if (n_steps == 0 && !(flags & FDTD_FWD_CHECK_FINITE)) return FDTD_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n_steps > 0) k_set_step<<<1, 1, 0, st>>>(p->d_t, t0);
    float* Hcur = b->H;
    float* Hnext = p->need_hprev ? p->h_twin : b->H;
    int done = 0;
    const bool use_graph = (flags & FDTD_FWD_GRAPH) != 0;
    const int unit = p->need_hprev ? 2 : 1;
    if (use_graph && n_steps >= 8) {
        int G = std::min(n_steps, 64);
        G -= G % unit;
        const bool same = p->gexec && p->gsteps == G && std::memcmp(&p->gbufs, b, sizeof(FdtdBuffers)) == 0;
        if (!same) {
            if (p->gexec) { cudaGraphExecDestroy(p->gexec); p->gexec = nullptr; }
            if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
            if (!p->cap_stream) {
                cudaError_t e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
                if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamCreate");
            }
            cudaError_t e = cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamBeginCapture");
            float* hc = b->H;
            float* hn = p->need_hprev ? p->h_twin : b->H;
            for (int s = 0; s < G; ++s) {
                launch_forward_step(p, b, hc, hn, p->cap_stream);
                if (p->need_hprev) std::swap(hc, hn);
            }
            e = cudaStreamEndCapture(p->cap_stream, &p->graph);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&p->gexec, p->graph, 0);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaGraphInstantiate");
            p->gbufs = *b;
            p->gsteps = G;
        }
        while (n_steps - done >= G) {
            cudaError_t e = cudaGraphLaunch(p->gexec, st);
            if (e != cudaSuccess) return cuda_fail(p, e, "cudaGraphLaunch");
            done += G;
        }
    }
    for (; done < n_steps; ++done) {
        launch_forward_step(p, b, Hcur, Hnext, st);
        if (p->need_hprev) std::swap(Hcur, Hnext);
    }
    if (p->need_hprev && Hcur != b->H) {
        cudaError_t e = cudaMemcpyAsync(b->H, Hcur, sizeof(float) * 3 * p->parts * p->g.N, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(p, e, "cudaMemcpyAsync");
    }
    if (flags & FDTD_FWD_CHECK_FINITE) {
        const long long n = 3 * p->parts * p->g.N;
        const int blocks = std::max(1, std::min(p->sm_count * 8, (int)((n + 255) / 256)));
        k_check_finite<<<blocks, 256, 0, st>>>(b->E, n, p->d_err);
        k_check_finite<<<blocks, 256, 0, st>>>(b->H, n, p->d_err);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_forward launch");
    return FDTD_OK;
}

// Reverse steps (fdtdx/fdtd/backward.py:62-135 with reset_fields=False and no
// detectors, the form the reversible gradient uses): per step t = t_end-1 ... :
// re-impose the recorded interfaces of step t, reverse H (sources subtracted first,
// psi frozen), reverse E.
int fdtd_reverse(FdtdPlan* p, const FdtdBuffers* b, int32_t t_end, int32_t n_steps, void* stream) {
    NvtxRange nvtx_range("fdtd_reverse");
    if (!p) return FDTD_EINVAL;
    if (cudaError_t pre = cudaGetLastError(); pre != cudaSuccess)
        return cuda_fail(p, pre, "error left pending by an earlier CUDA call (before fdtd_reverse)");
    if (int rc = check_bufs(p, b)) return rc;
    if (n_steps < 0 || t_end - n_steps < -1 || t_end > p->d.n_steps_total)
        return fail(p, FDTD_EINVAL, "reverse steps out of the range covered by the plan's tables");
    if (p->d.n_poles > 0) return fail(p, FDTD_EINVAL, "reverse steps of dispersive materials are not supported");
    if (n_steps == 0) return FDTD_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    k_set_step<<<1, 1, 0, st>>>(p->d_t, t_end - 1);
    for (int s = 0; s < n_steps; ++s) {
        interfaces<true>(p, b, b->H, st);
        launch_sources(p, b, false, b->H, 1, st);
        launch_side<true, true>(p, b, b->E, b->H, b->H, st);
        launch_sources(p, b, true, b->E, 1, st);
        launch_side<true, false>(p, b, b->H, b->E, b->E, st);
        k_advance<<<1, 1, 0, st>>>(p->d_t, -1);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_reverse launch");
    return FDTD_OK;
}

int64_t fdtd_footprint_bytes(const FdtdDesc* d) {
    if (!d) return -1;
    const long long N = (long long)d->nx * d->ny * d->nz;
    const int parts = d->bloch_axes ? 2 : 1;
    long long bytes = 4ll * N * (3 * parts + 3 * parts + d->n_eps + d->n_mu + d->n_sigma_E + d->n_sigma_H);
    if (d->n_eps == 9 || d->n_mu == 9 || d->n_sigma_E == 9 || d->n_sigma_H == 9) bytes += 24ll * parts * N;  // K and T
    if (d->n_poles > 0) bytes += 4ll * N * d->n_poles * (6 + 3 * d->n_disp);  // P pair and c1..c3
    const int n3[3] = {d->nx, d->ny, d->nz};
    long long iface = 0, psi = 0;
    for (int s = 0; s < d->n_slabs; ++s) {
        const FdtdSlabDesc& sl = d->slabs[s];
        psi += 4ll * 4 * parts * (N / n3[sl.axis]) * sl.thickness;  // psi_E and psi_H pairs
        iface += N / n3[sl.axis];
    }
    bytes += psi;
    // a recording plan is a reversible-gradient job: the state's cotangents, their twins, a
    // reconstruction copy of the state and the material gradients (inv_eps, and inv_mu when
    // the permeability is an array)
    if (d->record_interfaces) bytes += 3 * (24ll * N + psi) + 4ll * (d->n_eps + d->n_mu) * N;
    bool hprev = false;
    for (int q = 0; q < d->n_detectors; ++q) {
        const FdtdDetectorDesc& dd = d->detectors[q];
        const long long R = (long long)(dd.hi[0] - dd.lo[0]) * (dd.hi[1] - dd.lo[1]) * (dd.hi[2] - dd.lo[2]);
        const int C = popcount6(dd.comp_mask);
        long long on = 0;
        if (dd.slot)
            for (int t = 0; t < d->n_steps_total + 2; ++t) on = std::max<long long>(on, dd.slot[t] + 1);
        if (dd.kind == FDTD_DET_PHASOR) bytes += 8ll * dd.n_freq * C * (dd.reduce_volume ? 1 : R);
        else if (dd.kind == FDTD_DET_FIELD) bytes += 4ll * on * C * (dd.reduce_volume ? 1 : R);
        else bytes += 4ll * on * (dd.keep_all ? 3 : 1) * (dd.reduce_volume ? 1 : R);
        if (det_needs_h(dd)) hprev = true;
    }
    if (hprev) bytes += 12ll * parts * N;
    if (d->record_interfaces) bytes += (long long)rec_elem_bytes(d->recording_dtype) * 6 * parts * iface * rec_rows(*d);
    bytes += 1ll << 20;  // tables and scratch
    return bytes;
}

}  // extern "C"

#include "fdtd_adjoint_host.cuh"

extern "C" int fdtd_profile_forward(FdtdPlan* p, const FdtdBuffers* b, int32_t t0, int32_t n_steps, float* out_ms,
                                    void* stream) {
    if (p && p->parts != 1) return fail(p, FDTD_EINVAL, "per-launch profiling of complex (Bloch) fields is not supported");
    if (p && (p->full_e || p->full_h))
        return fail(p, FDTD_EINVAL, "per-launch profiling of full 3x3 tensor materials is not supported");
    if (p && p->d.n_poles > 0) return fail(p, FDTD_EINVAL, "per-launch profiling of dispersive materials is not supported");
    if (!p || !out_ms) return FDTD_EINVAL;
    if (int rc = check_bufs(p, b)) return rc;
    if (n_steps <= 0 || t0 < 0 || (long long)t0 + n_steps > (long long)p->d.n_steps_total + 1)
        return fail(p, FDTD_EINVAL, "time steps out of range");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaEvent_t ev[9];
    for (auto& e : ev) cudaEventCreate(&e);
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    k_set_step<<<1, 1, 0, st>>>(p->d_t, t0);
    float* Hcur = b->H;
    float* Hnext = p->need_hprev ? p->h_twin : b->H;
    for (int s = 0; s < n_steps; ++s) {
        cudaEventRecord(ev[0], st);
        launch_half<false, false>(p, make_upd(p, b, true, Hcur, b->E, b->E), st, ev[1]);
        cudaEventRecord(ev[2], st);
        launch_sources(p, b, true, b->E, 0, st);
        cudaEventRecord(ev[3], st);
        launch_half<false, true>(p, make_upd_fwd_H(p, b, Hcur, Hnext), st, ev[4]);
        cudaEventRecord(ev[5], st);
        launch_sources(p, b, false, Hnext, 0, st);
        cudaEventRecord(ev[6], st);
        DetFields f{b->E, Hcur, Hnext, b->inv_eps, p->d.n_eps, p->d.n_mu ? b->inv_mu : nullptr, p->d.n_mu ? p->d.n_mu : 1,
                    p->d.inv_mu_scalar};
        for (int q = 0; q < p->d.n_detectors; ++q) {
            if (p->fused[q]) continue;
            const DDet& dd = p->det[q];
            k_detector<<<dd.nblocks, kDetBlock, 0, st>>>(p->g, dd, p->d_t, f, b->det_state[q]);
            if (dd.reduce) k_detector_finalize<<<1, kDetBlock, 0, st>>>(dd, p->d_t, b->det_state[q]);
        }
        cudaEventRecord(ev[7], st);
        if (p->d.record_interfaces) interfaces<false>(p, b, Hnext, st);
        k_advance<<<1, 1, 0, st>>>(p->d_t, 1);
        cudaEventRecord(ev[8], st);
        cudaError_t e = cudaEventSynchronize(ev[8]);
        if (e != cudaSuccess) {
            for (auto& x : ev) cudaEventDestroy(x);
            return cuda_fail(p, e, "fdtd_profile_forward");
        }
        for (int k = 0; k < 8; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            acc[k] += ms;
        }
        if (p->need_hprev) std::swap(Hcur, Hnext);
    }
    if (p->need_hprev && Hcur != b->H)
        cudaMemcpyAsync(b->H, Hcur, sizeof(float) * 3 * p->g.N, cudaMemcpyDeviceToDevice, st);
    for (auto& x : ev) cudaEventDestroy(x);
    for (int k = 0; k < 8; ++k) out_ms[k] = (float)(acc[k] / n_steps);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_profile_forward");
    return FDTD_OK;
}

extern "C" int fdtd_plan_tune(FdtdPlan* p, int32_t chunk, int32_t vec) {
    if (!p) return FDTD_EINVAL;
    if (chunk <= 0) chunk = default_chunk(p->g.nx, p->g.ny, p->g.nz, p->sm_count);
    if (chunk > p->g.nx) chunk = p->g.nx;
    if (vec <= 0) vec = pick_vec(p->g.nz);
    if ((vec != 1 && vec != 2 && vec != 4) || p->g.nz % vec) return fail(p, FDTD_EINVAL, "vec must be 1, 2 or 4 and divide nz");
    if (chunk != p->chunk || vec != p->vec) {
        p->chunk = chunk;
        p->vec = vec;
        drop_graphs(p);
    }
    return FDTD_OK;
}

extern "C" int fdtd_plan_tune_shell(FdtdPlan* p, int32_t chunk, int32_t vec) {
    if (!p) return FDTD_EINVAL;
    if (chunk <= 0) chunk = kShellChunk;
    if (vec <= 0) vec = 1;
    if ((vec != 1 && vec != 2 && vec != 4) || (vec > 1 && p->g.nz % 4))
        return fail(p, FDTD_EINVAL, "shell vec must be 1, or 2 / 4 with nz % 4 == 0");
    if (chunk != p->shell_chunk || vec != p->shell_vec) {
        p->shell_chunk = chunk;
        p->shell_vec = vec;
        drop_graphs(p);
    }
    return FDTD_OK;
}

extern "C" int32_t fdtd_plan_chunk(const FdtdPlan* p) { return p ? p->chunk : 0; }
extern "C" int32_t fdtd_plan_vec(const FdtdPlan* p) { return p ? p->vec : 0; }

extern "C" int fdtd_plan_tune_tma(FdtdPlan* p, int32_t enable, int32_t tz, int32_t ty, int32_t stages, int32_t chunk) {
    if (!p) return FDTD_EINVAL;
    if (enable && !p->tma_ok) return fail(p, FDTD_EINVAL, "this scene cannot use the TMA kernels (periodic axis or nz % 4 != 0)");
    if (tz <= 0) {
        const Split sp = split_boxes(p);
        tz = pick_tz(sp.split ? sp.core.hi[2] - sp.core.lo[2] : p->g.nz);
    }
    if (ty <= 0) ty = 8;
    if (stages <= 0) stages = 4;
    if (tz % 4 || tz < 8 || tz > 120 || ty < 1 || ty * tz / 2 > 256 || stages < 2 || stages > kMaxStages)
        return fail(p, FDTD_EINVAL, "invalid TMA tile (tz a multiple of 4 in [8, 120], ty*tz/2 <= 256, 2..6 stages)");
    p->tma_tz = tz;
    p->tma_ty = ty;
    p->tma_ns = stages;
    if (enable) {
        configure_tma(p);
        if (!p->use_tma) return fail(p, FDTD_EINVAL, "TMA configuration does not fit the device");
        if (chunk > 0) p->tma_chunk = p->tma_chunk_e = std::min(chunk, p->g.nx);
    } else {
        p->use_tma = false;
    }
    drop_graphs(p);
    return FDTD_OK;
}

extern "C" int32_t fdtd_plan_uses_tma(const FdtdPlan* p) { return p && p->use_tma ? 1 : 0; }

extern "C" int fdtd_plan_tune_shell_tma(FdtdPlan* p, int32_t mode, int32_t tz, int32_t chunk) {
    if (!p) return FDTD_EINVAL;
    if (mode < 0 || mode > 5 || tz < 0 || tz % 4 || tz > 120 || chunk < 0)
        return fail(p, FDTD_EINVAL, "invalid slab-cell mode (0 to 5) or tile (tz a multiple of 4, <= 120)");
    p->shell_tma = mode;
    p->m2_tz = tz;
    configure_tma(p);
    if (shell_tma_mode(p) != mode) {
        p->shell_tma = shell_tma_mode(p);
        return fail(p, FDTD_EINVAL, "the CPML slab cells cannot run on the TMA kernels in this mode here (no TMA "
                                    "core, two slabs on a face or a tile that does not fit)");
    }
    if (chunk > 0) {
        if (mode == 1) p->m1_chunk = p->m1_chunk_e = std::min(chunk, p->g.nx);
        if (mode == 2) p->m2_chunk = p->m2_chunk_e = std::min(chunk, p->g.nx);
        if (mode == 3) p->m3_chunk = p->m3_chunk_e = std::min(chunk, p->g.nx);
        if (mode == 4 || mode == 5) p->m4_chunk = p->m4_chunk_e = std::min(chunk, p->g.nx);
        if (mode == 5) p->m3_chunk = p->m3_chunk_e = std::min(chunk, p->g.nx);
    }
    drop_graphs(p);
    return FDTD_OK;
}

extern "C" int32_t fdtd_plan_shell_tma(const FdtdPlan* p) { return p ? shell_tma_mode(p) : 0; }

extern "C" int fdtd_plan_status(FdtdPlan* p) {
    if (!p) return FDTD_EINVAL;
    int h = 0;
    cudaError_t e = cudaMemcpy(&h, p->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p, e, "fdtd_plan_status");
    if (h) {
        cudaMemset(p->d_err, 0, sizeof(int));
        if (h == FDTD_ENONFINITE)
            return fail(p, h, "a field holds a NaN or an infinity after the steps (check the materials, the sources "
                              "and the Courant number)");
        return fail(p, h, "a pipeline wait in a kernel ran out (the step's results are invalid)");
    }
    return FDTD_OK;
}

extern "C" int fdtd_debug_inject(int32_t kind, int32_t count) {
    if (count < 0) return FDTD_EINVAL;
    if (kind == FDTD_INJECT_ALLOC) g_inject_alloc.store(count);
    else if (kind == FDTD_INJECT_WAIT_EXPIRY) g_inject_expiry.store(count);
    else if (kind == FDTD_INJECT_BARRIER_EXPIRY) g_inject_barrier.store(count);
    else return FDTD_EINVAL;
    return FDTD_OK;
}
#include "fdtd_noalloc.cuh"
#include "fdtd_batch.cuh"
