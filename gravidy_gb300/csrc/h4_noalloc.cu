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
// they keep the contents of the last call: a kernel at the start of every
// call clears the control block (active count, work-queue head, error word
// and failing check site), and the partial sums are fully written before
// they are read.  Calls that overlap on the GPU (on different streams, or
// from different host threads, on one device) race on the arrays and must be
// serialised by the caller.
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/gravidy_gb300.h"
#include "h4_internal.cuh"

using namespace h4;

namespace {

constexpr size_t SCRATCH_DOUBLES = H4_NOALLOC_SCRATCH_DOUBLES;
constexpr unsigned MAX_N = 1u << 28;   // the particle limit of h4_create

static __device__ __align__(256) double g_noalloc_part[SCRATCH_DOUBLES];
static __device__ __align__(256) H4Ctrl g_noalloc_ctrl;

constexpr int MAX_DEVICES = 64;
int g_num_sms[MAX_DEVICES];   // SM count per device, 0 until the device's first call
std::mutex g_setup_mutex;

thread_local char g_err[256];

int noalloc_fail(int status, const char *msg, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess)
        snprintf(g_err, sizeof(g_err), "h4_forces_noalloc: %s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(g_err, sizeof(g_err), "h4_forces_noalloc: %s", msg);
    return status;
}

struct NoallocDevice {
    double *part;   // device address of g_noalloc_part
    H4Ctrl *ctrl;   // device address of g_noalloc_ctrl
    int num_sms;
};

// With device `dev` current: the device addresses of the file-scope arrays.
// In host code the array names are host-side stand-ins, not device
// addresses, so a kernel is only ever given these.  The first call on a
// device is its set-up (the look-up loads this file's device code there if
// it is not loaded yet, and the SM count is read once).  The look-up is
// repeated on every call -- it is cheap once the code is loaded -- so that a
// context created anew after cudaDeviceReset never gets a stale address.
int device_arrays(int dev, NoallocDevice *out) {
    if (dev < 0 || dev >= MAX_DEVICES) return noalloc_fail(H4_ERR_UNSUPPORTED, "device ordinal too large");
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_part);
    if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "cudaGetSymbolAddress(scratch)", e);
    out->part = (double *)p;
    e = cudaGetSymbolAddress(&p, g_noalloc_ctrl);
    if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "cudaGetSymbolAddress(control)", e);
    out->ctrl = (H4Ctrl *)p;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_num_sms[dev] == 0) {
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "cudaDeviceGetAttribute", e);
        g_num_sms[dev] = sms;
    }
    out->num_sms = g_num_sms[dev];
    return H4_OK;
}

// Start of a call: the control block the force kernel and the reduction
// read, cleared of the previous call's contents.
__global__ void k_noalloc_begin(H4Ctrl *c, unsigned nact) {
    c->nact = nact;
    c->work_next = 0u;
    c->err = 0u;
    c->bounds_site = 0u;
}

}  // namespace

extern "C" int h4_forces_noalloc(unsigned int n, double e2, const h4_double4 *d_pr, const h4_double4 *d_pv,
                                 unsigned int nact, const unsigned int *d_move, h4_forces *d_out,
                                 void *stream) {
    g_err[0] = 0;
    if (n < 1 || n > MAX_N) return noalloc_fail(H4_ERR_ARG, "n must be in [1, 2^28]");
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
    NoallocDevice nd{};
    int st = device_arrays(dev, &nd);
    if (st != H4_OK) return st;

    H4Dev d{};
    d.n = (int)n;
    d.n_pad = (int)n;
    d.e2 = e2;
    d.pr = (dbl4 *)d_pr;
    d.pv = (dbl4 *)d_pv;
    d.move = (unsigned *)d_move;
    d.part = nd.part;
    d.part_cap = SCRATCH_DOUBLES;
    d.ctrl = nd.ctrl;
    cudaStream_t s = (cudaStream_t)stream;
    k_noalloc_begin<<<1, 1, 0, s>>>(nd.ctrl, nact);
    launch_force_fp64(d, force_fp64_grid_warps(nd.num_sms), s);
    launch_reduce_to(d, (double *)d_out, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "kernel launch", e);
    if (kBoundsCheck) {   // bounds-checked build: wait and read the error word
        H4Ctrl c;
        e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = cudaMemcpy(&c, nd.ctrl, sizeof(c), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return noalloc_fail(H4_ERR_CUDA, "control block", e);
        if (c.err & H4_ERRBIT_BOUNDS) return noalloc_fail(H4_ERR_STATE, "bounds check failed");
    }
    return H4_OK;
}

extern "C" const char *h4_forces_noalloc_error(void) { return g_err; }
