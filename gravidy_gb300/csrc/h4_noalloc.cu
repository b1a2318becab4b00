// Force sum that allocates nothing (h4_forces_noalloc, include/gravidy_gb300.h).
//
// Some callers cannot call cudaMalloc: an application that reserves the GPU's
// memory for its own pool at start-up (a further cudaMalloc would fail or
// fragment that pool), or a time-critical loop that cannot take the device
// synchronisation cudaMalloc/cudaFree may imply.  They pass device buffers for
// the inputs and the output; the j-split partial sums and the work-queue
// counters that the FP64 force kernel needs live in file-scope device arrays
// of fixed size instead of the per-handle allocation.
//
// The arrays exist on every GPU where this library's device code is loaded
// and stay allocated until the process exits.  All calls share them, and
// they keep the contents of the last call: the control block is cleared by a
// kernel at the start of every call, and the partial sums are fully written
// before they are read.  Calls that overlap on the GPU (on different streams,
// or from different host threads, on one device) race on the arrays and must
// be serialised by the caller.
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/gravidy_gb300.h"
#include "h4_internal.cuh"

using namespace h4;

namespace {

constexpr size_t SCRATCH_DOUBLES = H4_NOALLOC_SCRATCH_DOUBLES;

static __device__ __align__(256) double g_noalloc_part[SCRATCH_DOUBLES];
static __device__ __align__(256) H4Ctrl g_noalloc_ctrl;

constexpr int MAX_DEVICES = 64;
struct NoallocDevice {
    bool ready = false;
    double *part = nullptr;   // device address of g_noalloc_part
    H4Ctrl *ctrl = nullptr;   // device address of g_noalloc_ctrl
    int num_sms = 0;
};
NoallocDevice g_devices[MAX_DEVICES];
std::mutex g_setup_mutex;

thread_local char g_err[256];

int noalloc_fail(int status, const char *msg, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess)
        snprintf(g_err, sizeof(g_err), "h4_forces_noalloc: %s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(g_err, sizeof(g_err), "h4_forces_noalloc: %s", msg);
    return status;
}

// Once per device, with that device current: the device addresses of the
// file-scope arrays.  In host code the array names are host-side stand-ins,
// not device addresses, so a kernel is only ever given these addresses.
int setup_device(int dev, NoallocDevice **out) {
    if (dev < 0 || dev >= MAX_DEVICES) return noalloc_fail(H4_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    NoallocDevice &nd = g_devices[dev];
    if (!nd.ready) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_part);
        if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "cudaGetSymbolAddress(scratch)", e);
        nd.part = (double *)p;
        e = cudaGetSymbolAddress(&p, g_noalloc_ctrl);
        if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "cudaGetSymbolAddress(control)", e);
        nd.ctrl = (H4Ctrl *)p;
        e = cudaDeviceGetAttribute(&nd.num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "cudaDeviceGetAttribute", e);
        nd.ready = true;
    }
    *out = &nd;
    return H4_OK;
}

}  // namespace

extern "C" int h4_forces_noalloc(unsigned int n, double e2, const h4_double4 *d_pr, const h4_double4 *d_pv,
                                 unsigned int nact, const unsigned int *d_move, h4_forces *d_out,
                                 void *stream) {
    g_err[0] = 0;
    if (n < 1) return noalloc_fail(H4_ERR_ARG, "n must be >= 1");
    if (nact == 0) return H4_OK;
    if (nact > H4_NOALLOC_MAX_NACT)
        return noalloc_fail(H4_ERR_ARG, "nact exceeds H4_NOALLOC_MAX_NACT (scratch is fixed-size)");
    if (nact > n) return noalloc_fail(H4_ERR_ARG, "nact larger than n");
    if (!d_pr || !d_pv || !d_move || !d_out) return noalloc_fail(H4_ERR_ARG, "null device pointer");
    if (((uintptr_t)d_pr | (uintptr_t)d_pv) % 32 != 0)
        return noalloc_fail(H4_ERR_ARG, "d_pr and d_pv must be 32-byte aligned");
    if ((uintptr_t)d_out % 8 != 0 || (uintptr_t)d_move % 4 != 0)
        return noalloc_fail(H4_ERR_ARG, "misaligned d_out or d_move");
    if (!(e2 >= 0.0)) return noalloc_fail(H4_ERR_ARG, "e2 must be >= 0");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "cudaGetDevice", e);
    NoallocDevice *nd = nullptr;
    int st = setup_device(dev, &nd);
    if (st != H4_OK) return st;

    H4Dev d{};
    d.n = (int)n;
    d.n_pad = (int)n;
    d.e2 = e2;
    d.pr = (dbl4 *)d_pr;
    d.pv = (dbl4 *)d_pv;
    d.move = (unsigned *)d_move;
    d.part = nd->part;
    d.part_cap = SCRATCH_DOUBLES;
    d.ctrl = nd->ctrl;
    cudaStream_t s = (cudaStream_t)stream;
    launch_set_nact(d, nact, s);   // nact, and the work-queue head back to zero
    launch_force_fp64(d, force_fp64_grid_warps(nd->num_sms), s);
    launch_reduce_to(d, (double *)d_out, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "kernel launch", e);
    if (kBoundsCheck) {   // bounds-checked build: wait and read the error word
        H4Ctrl c;
        e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = cudaMemcpy(&c, nd->ctrl, sizeof(c), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "control block", e);
        if (c.err & H4_ERRBIT_BOUNDS) return noalloc_fail(H4_ERR_STATE, "bounds check failed");
    }
    return H4_OK;
}

extern "C" const char *h4_forces_noalloc_error(void) { return g_err; }
