// Allocation-free variant of the A.X product (tincr_tda_products_noalloc).
//
// Some callers cannot let the library allocate device memory per call: a host that owns the
// whole GPU through its own pool or arena allocator (for instance a molecular-dynamics driver that
// evaluates excited-state forces every step, or an FMO driver running many monomer instances
// side by side), and callers for which the implicit device-wide synchronisation of cudaFree is
// not acceptable in the middle of their stream of work.  This entry point takes the trial vectors
// and the result as caller-owned device buffers and keeps its temporary AO-basis matrices (H, F,
// G and the Coulomb diagonals of the product, see tda.cu) in one file-scope device array of fixed
// size, so it calls no cudaMalloc, cudaFree or allocating library routine.
//
// A __device__ array exists once per CUDA context: every call made in the same context (normally
// the device's primary context, which all tincr contexts on that device share) uses the same
// array, and it keeps the contents of the last call.  Nothing in it has to start at zero (every
// element a call reads was written by that same call).  Calls in one CUDA context whose GPU work
// overlaps (from several host threads, or from several tincr contexts on the same GPU) race on it
// and must be serialised by the caller.
//
// Ordering: the product runs on the tincr context's own (non-blocking) stream.  It first makes that
// stream wait for all work queued so far on the legacy default stream (and so on every blocking
// stream), and it synchronises its own stream before returning.  Work that writes X_dev, or still
// uses AX_dev, on a non-blocking stream of the caller must be complete before the call.
#include "gemm_f64.cuh"
#include "kernels.cuh"
#include "ops.cuh"
#include "tda.cuh"

namespace tincr {

// 4 Mi doubles = 32 MiB, held by every GPU that loads the library until the process exits.
constexpr size_t NOALLOC_SCRATCH_DOUBLES = size_t(4) << 20;
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

// Device address of the scratch array in the current CUDA context, looked up at the first call on
// each tincr context, with that context's device current (the symbol's host-side name is only a
// stand-in and must never be handed to a kernel).  A tincr context lives in one CUDA context, so the
// cached address stays valid for as long as the tincr context does.
static double *scratch_of(Ctx &c) {
    if (!c.noalloc_scratch) {
        int cur = -1;
        TINCR_CUDA(cudaGetDevice(&cur));
        if (cur != c.device) fail(TINCR_BAD_ARG, "noalloc: the context's device is not current");
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            fail(TINCR_CUDA_ERR, std::string("noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        c.noalloc_scratch = static_cast<double *>(p);
    }
    return c.noalloc_scratch;
}

// A caller buffer must be device (or managed) memory of the context's device: a host pointer handed
// to the kernels would fault the GPU instead of failing the call.
static void check_device_pointer(const Ctx &c, const void *p, const char *what) {
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();   // clear the error this query recorded
        fail(TINCR_BAD_ARG, std::string("noalloc: ") + what + " is not a CUDA pointer");
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
        fail(TINCR_BAD_ARG, std::string("noalloc: ") + what + " is not device memory");
    if (a.type == cudaMemoryTypeDevice && a.device != c.device)
        fail(TINCR_BAD_ARG, std::string("noalloc: ") + what + " lives on another device");
}

// Scratch doubles needed for one trial vector: H and G (2n x v), F (2n x 2n, with exchange),
// d3, d2, z (n each).
static size_t noalloc_need(const Ctx &c) {
    size_t n = (size_t)c.n_orb, v = (size_t)c.n_virt;
    size_t need = 4 * n * v + 3 * n;
    if (c.lc) need += 4 * n * n;
    return need;
}

void products_noalloc(Ctx &c, int k, const double *X, double *AX) {
    if (!c.ready) fail(TINCR_BAD_ARG, "noalloc: tincr_tda_setup must be called first");
    if (k <= 0 || !X || !AX) fail(TINCR_BAD_ARG, "noalloc: bad arguments");
    const size_t need = noalloc_need(c);
    if (need > NOALLOC_SCRATCH_DOUBLES)
        fail(TINCR_BAD_ARG, "noalloc: system too large for the fixed scratch (needs " + std::to_string(need * 8) +
                                " bytes per trial vector, have " + std::to_string(NOALLOC_SCRATCH_DOUBLES * 8) + ")");
    if ((size_t)c.n_atoms * sizeof(double) > 48 * 1024) fail(TINCR_BAD_ARG, "noalloc: too many atoms");
    check_device_pointer(c, X, "X_dev");
    check_device_pointer(c, AX, "AX_dev");
    double *base = scratch_of(c);
    const int n = c.n_orb, o = c.n_occ, v = c.n_virt;
    const long long ov = c.ov;
    double *H = base, *G = H + 2LL * n * v, *d3 = G + 2LL * n * v, *d2 = d3 + n, *z = d2 + n, *F = z + n;
    cudaStream_t st = c.stream;
    // order after the work queued on the legacy default stream (which itself follows every blocking
    // stream); ev0 is free here: it only brackets the timed regions of the other entry points
    TINCR_CUDA(cudaEventRecord(c.ev0, cudaStreamLegacy));
    TINCR_CUDA(cudaStreamWaitEvent(st, c.ev0, 0));
    for (int b = 0; b < k; ++b) {
        const double *xb = X + (long long)b * ov;
        double *ab = AX + (long long)b * ov;
        // H = [Co; SCo] X
        gemm_f64<false, false>(st, 2 * n, v, o, c.dLst.p, o, 0, xb, v, 0, 1, EpiStore{H, 0, v, 1.0, 0.0});
        if (c.lc) {
            gemm_f64<false, true>(st, 2 * n, 2 * n, v, H, v, 0, c.dRv.p, v, 0, 1,
                                  EpiLcHadamard{F, c.d_glr_ao.p, d3, d2, n, -0.25});
        } else {
            dim3 g(ceil_div(2LL * n * 32, 256), 1);
            diag_dots_kernel<<<g, 256, 0, st>>>(n, v, H, v, 2LL * n * v, c.dRv.p, d3, d2);
            check_launch("diag_dots");
        }
        launch_coulomb(st, 1, n, c.n_atoms, c.d_ao_off.p, c.d_gamma.p, d3, d2, c.lc ? nullptr : z, c.lc ? F : nullptr,
                       nullptr, 1.0);
        if (c.lc) {
            gemm_f64<false, false>(st, 2 * n, v, 2 * n, F, 2 * n, 0, c.dRsw.p, v, 0, 1, EpiStore{G, 0, v, 1.0, 0.0});
        } else {
            dim3 g(ceil_div(2LL * n * v, 256), 1);
            scale_rows_kernel<<<g, 256, 0, st>>>(n, v, z, c.dRv.p, G);
            check_launch("scale_rows");
        }
        // AX = omega o X + [SCo; Co]^T G
        gemm_f64<true, false>(st, o, v, 2 * n, c.dLsw.p, o, 0, G, v, 0, 1, EpiOmega{ab, c.d_omega.p, xb, ov, v});
    }
    c.sync();
}

}  // namespace tincr
