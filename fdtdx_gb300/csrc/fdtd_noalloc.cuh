// fdtd_detector_sample_noalloc: a reduced detector sample that allocates nothing (included
// by fdtd_plan.cu, after the detector kernels it launches).
//
// Some callers cannot allocate device memory at the point where they want a detector
// value: an XLA FFI handler runs while XLA's allocator owns nearly all of HBM, so a
// cudaMalloc there competes with (or fails against) XLA's preallocated pool; a serving
// loop that admits jobs against a fixed HBM budget must not let a side query grow its
// footprint.  A plan cannot be built in either place either, since building one
// allocates its tables.  This entry point therefore runs the plan's own detector kernels
// (k_detector's reduce path and k_detector_finalize, unchanged) with their scratch (block
// partial sums, the step word and the slot table) in a file-scope static device array.
#pragma once

#include <mutex>

namespace {

constexpr int kNoAllocWords = 64;  // step word + slot table, read as int, all zero
constexpr int kNoAllocDevices = 64;

// [0, kNoAllocWords): int words (zero-initialised with the module, never written);
// [kNoAllocWords, +FDTD_NOALLOC_SCRATCH_FLOATS): block partial sums, written before read.
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocWords + FDTD_NOALLOC_SCRATCH_FLOATS];

std::mutex g_noalloc_mu;
float* g_noalloc_ptr[kNoAllocDevices] = {};

int noalloc_reject(const char* why) {
    fprintf(stderr, "fdtd_detector_sample_noalloc: %s\n", why);
    return FDTD_EINVAL;
}

}  // namespace

extern "C" int fdtd_detector_sample_noalloc(const FdtdDetectorDesc* det, int32_t nx, int32_t ny, int32_t nz,
                                            const int32_t periodic[3], const float* E, const float* H_prev,
                                            const float* H, const float* inv_eps, int32_t n_eps, const float* inv_mu,
                                            int32_t n_mu, float inv_mu_scalar, float* out, void* stream) {
    if (!det || !periodic || !E || !H || !out) return noalloc_reject("det, periodic, E, H and out are required");
    if (det->kind != FDTD_DET_FIELD && det->kind != FDTD_DET_FLUX && det->kind != FDTD_DET_ENERGY)
        return noalloc_reject("only FIELD, FLUX and ENERGY detectors are sampled");
    if (nx <= 0 || ny <= 0 || nz <= 0) return noalloc_reject("grid dimensions must be positive");
    const int n3[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a)
        if (det->lo[a] < 0 || det->hi[a] > n3[a] || det->lo[a] >= det->hi[a])
            return noalloc_reject("detector region must be non-empty and inside the grid");
    if (det->kind == FDTD_DET_FIELD && ((det->comp_mask & 63) == 0 || (det->comp_mask & ~63)))
        return noalloc_reject("comp_mask must select components among Ex..Hz");
    // H before the step's H update is read only where the plan's detectors read it too: exact
    // interpolation of a FLUX or ENERGY sample, or of a FIELD sample recording H components
    const bool needs_hprev = det->exact_interpolation &&
                             (det->kind != FDTD_DET_FIELD || (det->comp_mask & 56) != 0);
    if (needs_hprev && !H_prev)
        return noalloc_reject("H_prev is required with exact interpolation of H components");
    if (n_eps != 1 && n_eps != 3 && n_eps != 9) return noalloc_reject("n_eps must be 1, 3 or 9");
    if (n_mu != 0 && n_mu != 1 && n_mu != 3 && n_mu != 9) return noalloc_reject("n_mu must be 0, 1, 3 or 9");
    if (det->kind == FDTD_DET_ENERGY && (!inv_eps || (n_mu && !inv_mu)))
        return noalloc_reject("the energy sample needs inv_eps (and inv_mu when n_mu > 0)");

    DDet d{};
    d.kind = det->kind;
    d.comp_mask = det->kind == FDTD_DET_FIELD ? det->comp_mask : 63;
    d.exact = det->exact_interpolation ? 1 : 0;
    d.reduce = 1;
    d.inverse = 0;
    d.nfreq = 0;
    d.flux_axis = det->flux_axis;
    d.keep_all = det->keep_all;
    d.flux_sign = det->flux_sign;
    d.cell_weight = det->cell_weight;
    for (int a = 0; a < 3; ++a) { d.lo[a] = det->lo[a]; d.hi[a] = det->hi[a]; }
    d.rx = d.hi[0] - d.lo[0]; d.ry = d.hi[1] - d.lo[1]; d.rz = d.hi[2] - d.lo[2];
    d.R = (long long)d.rx * d.ry * d.rz;
    if (det->kind == FDTD_DET_FIELD) d.ncomp = popcount6(det->comp_mask);
    else if (det->kind == FDTD_DET_FLUX) d.ncomp = det->keep_all ? 3 : 1;
    else d.ncomp = 1;
    if (det->kind == FDTD_DET_FLUX && !det->keep_all && (det->flux_axis < 0 || det->flux_axis > 2))
        return noalloc_reject("flux_axis must be 0, 1 or 2");
    const long long nblocks = (d.R + kDetBlock - 1) / kDetBlock;
    if (nblocks * d.ncomp > FDTD_NOALLOC_SCRATCH_FLOATS) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "a region of %lld cells needs %lld partial sums; the static scratch holds %d "
                 "(at most %lld cells for %d component(s))",
                 d.R, nblocks * d.ncomp, FDTD_NOALLOC_SCRATCH_FLOATS,
                 (long long)(FDTD_NOALLOC_SCRATCH_FLOATS / d.ncomp) * kDetBlock, d.ncomp);
        return noalloc_reject(msg);
    }
    d.nblocks = (int)nblocks;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_reject(cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocDevices) return noalloc_reject("device ordinal beyond the scratch address table");
    // The scratch address is looked up again on every call made outside stream capture, so
    // a device reset (which reloads the module and may move the array) is picked up by the
    // next call; inside a capture the address of the last call on this device is used.
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusNone;
    }
    float* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) {
                fprintf(stderr, "fdtd_detector_sample_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
                return FDTD_ECUDA;
            }
            g_noalloc_ptr[dev] = static_cast<float*>(ptr);
        }
        base = g_noalloc_ptr[dev];
    }
    const int* words = reinterpret_cast<const int*>(base);
    const int* tp = words;        // step word: 0
    d.slot = words + 1;           // slot table: slot[tp + 1] = 0
    d.w = nullptr;
    d.partial = base + kNoAllocWords;

    Geo g{};
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.N = (long long)nx * ny * nz;
    g.px = periodic[0] != 0; g.py = periodic[1] != 0; g.pz = periodic[2] != 0;
    DetFields f{E, needs_hprev ? H_prev : H, H, inv_eps, n_eps, n_mu ? inv_mu : nullptr, n_mu ? n_mu : 1, inv_mu_scalar};
    k_detector<<<d.nblocks, kDetBlock, 0, st>>>(g, d, tp, f, out);
    k_detector_finalize<<<1, kDetBlock, 0, st>>>(d, tp, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "fdtd_detector_sample_noalloc: launch: %s\n", cudaGetErrorString(e));
        return FDTD_ECUDA;
    }
    return FDTD_OK;
}
