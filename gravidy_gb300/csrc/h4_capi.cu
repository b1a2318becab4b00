// C ABI of the Hermite4 block-step path (declarations: include/gravidy_gb300.h).
//
// Host-side owner of one system's device state: allocation, the order of
// kernel launches for each reference method, the CUDA graph of a whole block
// step with a device-side while loop, and status codes in place of the
// reference's exit-on-error (src/include/gpu/Hermite4GPU.cuh:43-50).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gravidy_gb300.h"
#include "h4_internal.cuh"

using namespace h4;

namespace {

thread_local std::string g_last_error;

int fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return H4_ERR_CUDA;
}

#define H4_TRY(call, what)                           \
    do {                                             \
        cudaError_t e__ = (call);                    \
        if (e__ != cudaSuccess) return cuda_fail(e__, what); \
    } while (0)

// Active-set size from which the tiled mixed kernel is used instead of the
// warp items.  Measured crossover of the two mixed kernels on GB300 (force kernel time,
// N = 32768 .. 2^20): the warp items win below about 700 active particles at
// N = 32768, 300 at N = 65536 and 160-250 at N = 262144 and 2^20.
unsigned default_mixed_threshold(unsigned n) { return n >= 131072u ? 192u : (n >= 65536u ? 320u : 768u); }

bool is_pow2(double x) {
    if (!(x > 0.0) || !std::isfinite(x)) return false;
    int ex;
    double m = std::frexp(x, &ex);
    return m == 0.5;
}

}  // namespace

// CUDA-event timers per phase, with the reference's phase names (Gtime,
// src/include/common.hpp:287-310): each phase keeps one pending event pair,
// resolved when the phase is issued again or when the totals are read.
enum Phase { PH_PREDICTION, PH_UPDATE, PH_GRAV, PH_CORRECTION, PH_ACTIVE, PH_NEXT, PH_ENERGY, PH_ADVANCE, PH_COUNT };
static const char *kPhaseNames[PH_COUNT] = {"prediction", "update", "grav", "correction", "active_set",
                                            "next_time", "energy", "advance"};
struct PhaseTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    bool pending = false;
    double total_ms = 0.0;
    unsigned long long count = 0;
};

struct h4_system_s {
    H4Dev d;
    int mode = H4_FORCE_FP64;
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    H4Ctrl *h_ctrl = nullptr;      // pinned host copy of the control block
    double *h_energy = nullptr;    // pinned [2]
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    float last_force_ms = 0.f, last_advance_ms = 0.f;
    unsigned long long launches = 0;
    bool forces_ready = false;
    // device-resident loop
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_mode = -1;
    unsigned mixed_threshold = 0;   // set at creation from N
    PhaseTimer phase[PH_COUNT];
    cudaStream_t graph_stream = nullptr;
};

namespace {

void free_device(h4_system_s *h) {
    H4Dev &d = h->d;
    void *ptrs[] = {d.r, d.v, d.f, d.old, d.a2, d.a3, d.t, d.dt, d.pr, d.pv, d.jf0, d.jf1, d.jf2, d.jd,
                    d.move, d.blk_cnt, d.part, d.epot_i, d.energy_out, d.ctrl};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->h_ctrl) cudaFreeHost(h->h_ctrl);
    if (h->h_energy) cudaFreeHost(h->h_energy);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    if (h->graph_stream) cudaStreamDestroy(h->graph_stream);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->ev2) cudaEventDestroy(h->ev2);
    if (h->ev3) cudaEventDestroy(h->ev3);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    for (auto &p : h->phase) {
        if (p.a) cudaEventDestroy(p.a);
        if (p.b) cudaEventDestroy(p.b);
    }
}

void phase_resolve(PhaseTimer &p) {
    if (!p.pending) return;
    if (cudaEventSynchronize(p.b) == cudaSuccess) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) p.total_ms += ms;
        p.count += 1;
    }
    p.pending = false;
}

// Timers are best effort: a timer whose events cannot be created stays off,
// and its failure is cleared so that it never surfaces as the error of the
// call it times.
void phase_begin(h4_system_s *h, Phase ph) {
    PhaseTimer &p = h->phase[ph];
    phase_resolve(p);
    if (!p.a) {
        if (cudaEventCreate(&p.a) != cudaSuccess || cudaEventCreate(&p.b) != cudaSuccess) {
            if (p.a) cudaEventDestroy(p.a);
            p.a = p.b = nullptr;
            cudaGetLastError();
            return;
        }
    }
    cudaEventRecord(p.a, h->stream);
}

void phase_end(h4_system_s *h, Phase ph) {
    PhaseTimer &p = h->phase[ph];
    if (!p.a) return;
    cudaEventRecord(p.b, h->stream);
    p.pending = true;
}

int grid_warps(const h4_system_s *h) { return force_fp64_grid_warps(h->num_sms); }

// Force sum of the active list on the device (nact in the control block),
// leaving partial sums in d.part.  known_nact < 0: count only on the device.
void launch_force(h4_system_s *h, cudaStream_t s, long long known_nact = -1) {
    switch (h->mode) {
    case H4_FORCE_EXACT: launch_force_exact(h->d, s); h->launches += 1; break;
    case H4_FORCE_MIXED:
        h->launches += launch_force_mixed(h->d, h->num_sms, h->mixed_threshold, known_nact, s);
        break;
    default: launch_force_fp64(h->d, grid_warps(h), s); h->launches += 1; break;
    }
}

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return H4_OK;
}

int sync_ctrl(h4_system_s *h) {
    H4_TRY(cudaMemcpyAsync(h->h_ctrl, h->d.ctrl, sizeof(H4Ctrl), cudaMemcpyDeviceToHost, h->stream),
           "copy control block");
    H4_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    if (h->h_ctrl->err & H4_ERRBIT_BOUNDS)   // bounds-checked build only
        return fail(H4_ERR_STATE, "bounds check failed at site " + std::to_string(h->h_ctrl->bounds_site));
    return H4_OK;
}

double bits_to_double_host(unsigned long long b) {
    double x;
    std::memcpy(&x, &b, sizeof(x));
    return x;
}

// One block step, device-driven (no host values): active set + predictor ->
// force -> reduce + save old + correct -> next time; inside the graph's loop
// (cond given) the next-time kernel also does the loop's bookkeeping.
void enqueue_step(h4_system_s *h, cudaStream_t s, const cudaGraphConditionalHandle *cond) {
    launch_find_active_predict(h->d, s);
    launch_force(h, s);
    launch_correct(h->d, false, 0.0, true, s);
    if (cond)
        launch_next_time_bookkeeping(h->d, *cond, s);
    else
        launch_next_time(h->d, false, s);
    h->launches += 4;   // active set + predictor (2 kernels), correct, next time
}

// Kernels in one captured block step (force kernels counted per mode).
int step_kernel_count(const h4_system_s *h) { return 4 + (h->mode == H4_FORCE_MIXED ? 2 : 1); }

int build_graph(h4_system_s *h) {
    if (h->graph_exec && h->graph_mode == h->mode) return H4_OK;
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; }
    if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
    if (!h->graph_stream) H4_TRY(cudaStreamCreateWithFlags(&h->graph_stream, cudaStreamNonBlocking), "graph stream");
    H4_TRY(cudaGraphCreate(&h->graph, 0), "cudaGraphCreate");
    cudaGraphConditionalHandle cond;
    H4_TRY(cudaGraphConditionalHandleCreate(&cond, h->graph, 1u, cudaGraphCondAssignDefault),
           "cudaGraphConditionalHandleCreate");
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    H4_TRY(cudaGraphAddNode(&node, h->graph, nullptr, nullptr, 0, &cp), "add while node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    H4_TRY(cudaStreamBeginCaptureToGraph(h->graph_stream, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal),
           "begin capture");
    unsigned long long saved = h->launches;
    enqueue_step(h, h->graph_stream, &cond);
    h->launches = saved;
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->graph_stream, &captured);
    if (e != cudaSuccess) return cuda_fail(e, "end capture");
    H4_TRY(cudaGraphInstantiate(&h->graph_exec, h->graph, 0), "cudaGraphInstantiate");
    h->graph_mode = h->mode;
    return H4_OK;
}

}  // namespace

extern "C" {

const char *h4_last_error(void) { return g_last_error.c_str(); }

const char *h4_status_string(int status) {
    switch (status) {
    case H4_OK: return "ok";
    case H4_ERR_ARG: return "invalid argument";
    case H4_ERR_CUDA: return "CUDA error";
    case H4_ERR_ALLOC: return "allocation failed";
    case H4_ERR_STATE: return "call out of order";
    case H4_ERR_NONFINITE: return "non-finite value in the state";
    case H4_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

int h4_abi_version(void) { return H4_ABI_VERSION; }

int h4_build_flags(void) { return kBoundsCheck ? H4_BUILD_BOUNDS_CHECK : 0; }

int h4_create(h4_handle *out, unsigned int n, double e2, float eta, const h4_double4 *r,
              const h4_double4 *v, int mode) {
    if (!out) return fail(H4_ERR_ARG, "h4_create: out is NULL");
    *out = nullptr;
    if (n < 1 || n > (1u << 28)) return fail(H4_ERR_ARG, "h4_create: n must be in [1, 2^28]");
    if (!r || !v) return fail(H4_ERR_ARG, "h4_create: r and v must not be NULL");
    if (!(e2 >= 0.0) || !std::isfinite(e2)) return fail(H4_ERR_ARG, "h4_create: e2 must be finite and >= 0");
    if (!(eta > 0.0f) || !std::isfinite(eta)) return fail(H4_ERR_ARG, "h4_create: eta must be > 0");
    if (mode < H4_FORCE_FP64 || mode > H4_FORCE_MIXED) return fail(H4_ERR_ARG, "h4_create: unknown force mode");
    for (unsigned i = 0; i < n; i++) {
        if (!std::isfinite(r[i].x) || !std::isfinite(r[i].y) || !std::isfinite(r[i].z) ||
            !std::isfinite(r[i].w) || !std::isfinite(v[i].x) || !std::isfinite(v[i].y) ||
            !std::isfinite(v[i].z))
            return fail(H4_ERR_NONFINITE, "h4_create: non-finite position, mass or velocity of particle " +
                                              std::to_string(i));
    }
    h4_system_s *h = new (std::nothrow) h4_system_s();
    if (!h) return fail(H4_ERR_ALLOC, "h4_create: host allocation");
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "h4_create: no CUDA device"); }
    H4Dev &d = h->d;
    d.n = (int)n;
    d.n_pad = (int)((n + 255u) & ~255u);
    d.e2 = e2;
    d.eta = (double)eta;
    d.dt_min = 1.1920928955078125e-07;
    d.dt_max = 0.125;
    h->mode = mode;
    d.mixed = mode == H4_FORCE_MIXED ? 1 : 0;
    h->mixed_threshold = default_mixed_threshold(n);
    const size_t N = n, NP = (size_t)d.n_pad;
    d.part_cap = 6 * (N + 262144);
    const int nflag = (int)((N + FLAG_CHUNK - 1) / FLAG_CHUNK);
    struct { void **p; size_t bytes; } allocs[] = {
        {(void **)&d.r, N * sizeof(dbl4)},       {(void **)&d.v, N * sizeof(dbl4)},
        {(void **)&d.f, N * 6 * sizeof(double)}, {(void **)&d.old, N * 6 * sizeof(double)},
        {(void **)&d.a2, N * 3 * sizeof(double)}, {(void **)&d.a3, N * 3 * sizeof(double)},
        {(void **)&d.t, N * sizeof(double)},     {(void **)&d.dt, N * sizeof(double)},
        {(void **)&d.pr, NP * sizeof(dbl4)},     {(void **)&d.pv, NP * sizeof(dbl4)},
        {(void **)&d.jf0, NP * sizeof(float4)},  {(void **)&d.jf1, NP * sizeof(float4)},
        {(void **)&d.jf2, NP * sizeof(float4)},  {(void **)&d.jd, 5 * NP * sizeof(float4)},
        {(void **)&d.move, N * sizeof(unsigned)}, {(void **)&d.blk_cnt, (size_t)nflag * sizeof(unsigned)},
        {(void **)&d.part, d.part_cap * sizeof(double)}, {(void **)&d.epot_i, N * sizeof(double)},
        {(void **)&d.energy_out, 2 * sizeof(double)}, {(void **)&d.ctrl, sizeof(H4Ctrl)},
    };
    for (auto &a : allocs) {
        e = cudaMalloc(a.p, a.bytes);
        if (e != cudaSuccess) { free_device(h); delete h; return fail(H4_ERR_ALLOC, std::string("h4_create: cudaMalloc: ") + cudaGetErrorString(e)); }
    }
    e = cudaMallocHost((void **)&h->h_ctrl, sizeof(H4Ctrl));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h->h_energy, 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev2);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev3);
    if (e != cudaSuccess) { free_device(h); delete h; return cuda_fail(e, "h4_create: setup"); }
    h->stream = h->own_stream;
    cudaStream_t s = h->stream;
    // r with the mass rounded to float (the reference parses masses as float,
    // NbodySystem.cpp:174); everything else zero as Hermite4::init_data.
    dbl4 *tmp = nullptr;
    e = cudaMallocHost((void **)&tmp, N * sizeof(dbl4) * 2);
    if (e != cudaSuccess) { free_device(h); delete h; return cuda_fail(e, "h4_create: staging"); }
    for (size_t i = 0; i < N; i++) {
        tmp[i] = make_dbl4(r[i].x, r[i].y, r[i].z, (double)(float)r[i].w);
        tmp[N + i] = make_dbl4(v[i].x, v[i].y, v[i].z, 0.0);
    }
    e = cudaMemcpyAsync(d.r, tmp, N * sizeof(dbl4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.v, tmp + N, N * sizeof(dbl4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.f, 0, N * 6 * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.old, 0, N * 6 * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.a2, 0, N * 3 * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.a3, 0, N * 3 * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.t, 0, N * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.dt, 0, N * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.move, 0, N * sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.ctrl, 0, sizeof(H4Ctrl), s);
    if (e == cudaSuccess) {
        launch_set_pred_from_state(d, s);
        launch_pad_predicted(d, s);
        h->launches += 2;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeHost(tmp);
    if (e != cudaSuccess) { free_device(h); delete h; return cuda_fail(e, "h4_create: upload"); }
    *out = h;
    return H4_OK;
}

int h4_destroy(h4_handle h) {
    if (!h) return H4_OK;
    cudaStreamSynchronize(h->stream);
    free_device(h);
    delete h;
    return H4_OK;
}

int h4_set_stream(h4_handle h, void *stream) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    H4_TRY(cudaStreamSynchronize(h->stream), "synchronize");
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return H4_OK;
}

int h4_set_dt_limits(h4_handle h, double dt_min, double dt_max) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    if (!is_pow2(dt_min) || !is_pow2(dt_max) || dt_min > dt_max)
        return fail(H4_ERR_ARG, "h4_set_dt_limits: bounds must be powers of two with dt_min <= dt_max");
    h->d.dt_min = dt_min;
    h->d.dt_max = dt_max;
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; h->graph_mode = -1; }
    return H4_OK;
}

int h4_set_force_mode(h4_handle h, int mode) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    if (mode < H4_FORCE_FP64 || mode > H4_FORCE_MIXED) return fail(H4_ERR_ARG, "unknown force mode");
    const int was_mixed = h->d.mixed;
    h->mode = mode;
    h->d.mixed = mode == H4_FORCE_MIXED ? 1 : 0;
    if (h->d.mixed && !was_mixed) {   // the FP32 j data of the current predictors
        launch_pack_j(h->d, h->stream);
        h->launches += 1;
        return check_launch("h4_set_force_mode");
    }
    return H4_OK;
}

int h4_set_mixed_threshold(h4_handle h, unsigned int nact_threshold) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    if (nact_threshold < 1) return fail(H4_ERR_ARG, "threshold must be >= 1");
    h->mixed_threshold = nact_threshold;
    if (h->graph_exec) { cudaGraphExecDestroy(h->graph_exec); h->graph_exec = nullptr; h->graph_mode = -1; }
    return H4_OK;
}

int h4_init_acc_jrk(h4_handle h) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    cudaStream_t s = h->stream;
    // Predictors = current state, as Hermite4::init_data leaves them before
    // the reference calls init_acc_jrk (Hermite4.cpp:202-214).
    launch_set_pred_from_state(h->d, s);
    launch_identity_move(h->d, s);
    h->launches += 1;
    cudaEventRecord(h->ev0, s);
    launch_force(h, s, (long long)h->d.n);
    cudaEventRecord(h->ev1, s);
    launch_reduce_forces(h->d, false, s);
    h->launches += 2;
    int st = check_launch("h4_init_acc_jrk");
    if (st) return st;
    H4_TRY(cudaEventSynchronize(h->ev1), "h4_init_acc_jrk");
    cudaEventElapsedTime(&h->last_force_ms, h->ev0, h->ev1);
    h->forces_ready = true;
    return H4_OK;
}

int h4_init_dt(h4_handle h, double *atime, float eta, double itime) {
    if (!h || !atime) return fail(H4_ERR_ARG, "h4_init_dt: null argument");
    if (!h->forces_ready) return fail(H4_ERR_STATE, "h4_init_dt: call h4_init_acc_jrk first");
    launch_init_dt(h->d, eta, itime, h->stream);
    h->launches += 2;
    int st = check_launch("h4_init_dt");
    if (st) return st;
    if ((st = sync_ctrl(h))) return st;
    const double m = bits_to_double_host(h->h_ctrl->atime_bits);
    if (m < *atime) *atime = m;
    launch_set_atime(h->d, *atime, h->stream);
    h->launches += 1;
    return check_launch("h4_init_dt");
}

int h4_find_particles_to_move(h4_handle h, double itime, unsigned int *nact) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    phase_begin(h, PH_ACTIVE);
    launch_find_active(h->d, true, itime, h->stream);
    phase_end(h, PH_ACTIVE);
    h->launches += 2;
    int st = check_launch("h4_find_particles_to_move");
    if (st) return st;
    if (nact) {
        if ((st = sync_ctrl(h))) return st;
        *nact = h->h_ctrl->nact;
    }
    return H4_OK;
}

static int set_nact(h4_system_s *h, unsigned nact) {
    if (nact > (unsigned)h->d.n) return fail(H4_ERR_ARG, "nact larger than n");
    launch_set_nact(h->d, nact, h->stream);
    h->launches += 1;
    return H4_OK;
}

int h4_save_old_acc_jrk(h4_handle h, unsigned int nact) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    int st = set_nact(h, nact);
    if (st) return st;
    launch_save_old(h->d, h->stream);
    h->launches += 1;
    return check_launch("h4_save_old_acc_jrk");
}

int h4_predicted_pos_vel(h4_handle h, double itime) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    phase_begin(h, PH_PREDICTION);
    launch_predict(h->d, true, itime, h->stream);
    phase_end(h, PH_PREDICTION);
    h->launches += 1;
    return check_launch("h4_predicted_pos_vel");
}

int h4_update_acc_jrk(h4_handle h, unsigned int nact) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    int st = set_nact(h, nact);
    if (st) return st;
    if (nact == 0) return H4_OK;
    phase_begin(h, PH_UPDATE);
    phase_begin(h, PH_GRAV);
    cudaEventRecord(h->ev0, h->stream);
    launch_force(h, h->stream, (long long)nact);
    cudaEventRecord(h->ev1, h->stream);
    phase_end(h, PH_GRAV);
    launch_reduce_forces(h->d, false, h->stream);
    phase_end(h, PH_UPDATE);
    h->launches += 1;
    return check_launch("h4_update_acc_jrk");
}

int h4_correction_pos_vel(h4_handle h, double itime, unsigned int nact) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    int st = set_nact(h, nact);
    if (st) return st;
    phase_begin(h, PH_CORRECTION);
    launch_correct(h->d, true, itime, false, h->stream);
    phase_end(h, PH_CORRECTION);
    h->launches += 1;
    return check_launch("h4_correction_pos_vel");
}

int h4_next_integration_time(h4_handle h, double *atime) {
    if (!h || !atime) return fail(H4_ERR_ARG, "h4_next_integration_time: null argument");
    phase_begin(h, PH_NEXT);
    launch_next_time(h->d, true, h->stream);
    phase_end(h, PH_NEXT);
    h->launches += 2;
    int st = check_launch("h4_next_integration_time");
    if (st) return st;
    if ((st = sync_ctrl(h))) return st;
    *atime = bits_to_double_host(h->h_ctrl->atime_bits);
    return H4_OK;
}

int h4_get_energy(h4_handle h, double *ekin, double *epot, double *etot) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    phase_begin(h, PH_ENERGY);
    launch_energy(h->d, h->stream);
    phase_end(h, PH_ENERGY);
    h->launches += 2;
    int st = check_launch("h4_get_energy");
    if (st) return st;
    H4_TRY(cudaMemcpyAsync(h->h_energy, h->d.energy_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
           "h4_get_energy copy");
    H4_TRY(cudaStreamSynchronize(h->stream), "h4_get_energy");
    if (ekin) *ekin = h->h_energy[0];
    if (epot) *epot = h->h_energy[1];
    if (etot) *etot = h->h_energy[0] + h->h_energy[1] + 0.0;
    return H4_OK;
}

int h4_step(h4_handle h, double *atime, double *itime, unsigned int *nact) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    if (!h->forces_ready) return fail(H4_ERR_STATE, "h4_step: call h4_init_acc_jrk and h4_init_dt first");
    if (atime) { launch_set_atime(h->d, *atime, h->stream); h->launches += 1; }
    enqueue_step(h, h->stream, nullptr);
    int st = check_launch("h4_step");
    if (st) return st;
    if (atime || itime || nact) {
        if ((st = sync_ctrl(h))) return st;
        if (atime) *atime = bits_to_double_host(h->h_ctrl->atime_bits);
        if (itime) *itime = h->h_ctrl->itime;
        if (nact) *nact = h->h_ctrl->nact;
        if (h->h_ctrl->err & H4_ERRBIT_NONFINITE) return fail(H4_ERR_NONFINITE, "h4_step: non-finite state");
    }
    return H4_OK;
}

int h4_advance(h4_handle h, double t_stop, double t_log, double *atime, double *itime, double stats[5]) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    if (!h->forces_ready) return fail(H4_ERR_STATE, "h4_advance: call h4_init_acc_jrk and h4_init_dt first");
    int st = build_graph(h);
    if (st) return st;
    cudaStream_t s = h->stream;
    // Control block: loop bounds and fresh counters; the next block time comes
    // from the caller when given.
    if ((st = sync_ctrl(h))) return st;
    H4Ctrl c = *h->h_ctrl;
    if (atime) c.atime_bits = 0, std::memcpy(&c.atime_bits, atime, sizeof(double));
    c.t_stop = t_stop;
    c.t_log = t_log;
    c.steps = c.psteps = c.inter = 0;
    c.running = 1;
    {
        const double t0 = atime ? *atime : bits_to_double_host(c.atime_bits);
        double span = (t_stop < t_log ? t_stop : t_log) - t0;
        if (!(span > 0.0)) span = 0.0;
        const double cap = span / h->d.dt_min + 16.0;
        c.max_steps = cap < 1.0e15 ? (unsigned long long)cap : 1000000000000000ull;
    }
    *h->h_ctrl = c;
    H4_TRY(cudaMemcpyAsync(h->d.ctrl, h->h_ctrl, sizeof(H4Ctrl), cudaMemcpyHostToDevice, s), "h4_advance ctrl");
    cudaEventRecord(h->ev2, s);
    H4_TRY(cudaGraphLaunch(h->graph_exec, s), "h4_advance graph launch");
    cudaEventRecord(h->ev3, s);
    if ((st = sync_ctrl(h))) return st;
    cudaEventElapsedTime(&h->last_advance_ms, h->ev2, h->ev3);
    h->phase[PH_ADVANCE].total_ms += h->last_advance_ms;
    h->phase[PH_ADVANCE].count += 1;
    const H4Ctrl &o = *h->h_ctrl;
    h->launches += (unsigned long long)o.steps * (unsigned long long)step_kernel_count(h);
    if (atime) *atime = bits_to_double_host(o.atime_bits);
    if (itime) *itime = o.itime;
    if (stats) {
        stats[0] = (double)o.steps;
        stats[1] = (double)o.psteps;
        stats[2] = (double)o.inter;
        stats[3] = o.itime;
        stats[4] = (double)o.nact;
    }
    if (o.err & H4_ERRBIT_NONFINITE) return fail(H4_ERR_NONFINITE, "h4_advance: non-finite state");
    if (o.err & H4_ERRBIT_STEPCAP) return fail(H4_ERR_STATE, "h4_advance: step bound reached");
    if (o.err & H4_ERRBIT_TIMEOUT) return fail(H4_ERR_CUDA, "h4_advance: a bounded device wait timed out");
    return H4_OK;
}

int h4_download(h4_handle h, h4_double4 *r, h4_double4 *v, h4_forces *f, h4_forces *old, h4_double3 *a2,
                h4_double3 *a3, double *t, double *dt, unsigned int *move) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    if (kBoundsCheck) {   // a failed check of the bounds-checked build surfaces here at the latest
        int st = sync_ctrl(h);
        if (st) return st;
    }
    const size_t N = h->d.n;
    cudaStream_t s = h->stream;
    if (r) H4_TRY(cudaMemcpyAsync(r, h->d.r, N * 32, cudaMemcpyDeviceToHost, s), "download r");
    if (v) H4_TRY(cudaMemcpyAsync(v, h->d.v, N * 32, cudaMemcpyDeviceToHost, s), "download v");
    if (f) H4_TRY(cudaMemcpyAsync(f, h->d.f, N * 48, cudaMemcpyDeviceToHost, s), "download f");
    if (old) H4_TRY(cudaMemcpyAsync(old, h->d.old, N * 48, cudaMemcpyDeviceToHost, s), "download old");
    if (a2) H4_TRY(cudaMemcpyAsync(a2, h->d.a2, N * 24, cudaMemcpyDeviceToHost, s), "download a2");
    if (a3) H4_TRY(cudaMemcpyAsync(a3, h->d.a3, N * 24, cudaMemcpyDeviceToHost, s), "download a3");
    if (t) H4_TRY(cudaMemcpyAsync(t, h->d.t, N * 8, cudaMemcpyDeviceToHost, s), "download t");
    if (dt) H4_TRY(cudaMemcpyAsync(dt, h->d.dt, N * 8, cudaMemcpyDeviceToHost, s), "download dt");
    if (move) H4_TRY(cudaMemcpyAsync(move, h->d.move, N * 4, cudaMemcpyDeviceToHost, s), "download move");
    H4_TRY(cudaStreamSynchronize(s), "download");
    return H4_OK;
}

int h4_upload(h4_handle h, const h4_double4 *r, const h4_double4 *v, const h4_forces *f, const h4_forces *old,
              const double *t, const double *dt) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    const size_t N = h->d.n;
    cudaStream_t s = h->stream;
    if (r) H4_TRY(cudaMemcpyAsync(h->d.r, r, N * 32, cudaMemcpyHostToDevice, s), "upload r");
    if (v) H4_TRY(cudaMemcpyAsync(h->d.v, v, N * 32, cudaMemcpyHostToDevice, s), "upload v");
    if (f) H4_TRY(cudaMemcpyAsync(h->d.f, f, N * 48, cudaMemcpyHostToDevice, s), "upload f");
    if (old) H4_TRY(cudaMemcpyAsync(h->d.old, old, N * 48, cudaMemcpyHostToDevice, s), "upload old");
    if (t) H4_TRY(cudaMemcpyAsync(h->d.t, t, N * 8, cudaMemcpyHostToDevice, s), "upload t");
    if (dt) H4_TRY(cudaMemcpyAsync(h->d.dt, dt, N * 8, cudaMemcpyHostToDevice, s), "upload dt");
    H4_TRY(cudaStreamSynchronize(s), "upload");
    if (f) h->forces_ready = true;
    return H4_OK;
}

int h4_restore(h4_handle h, const h4_double4 *r, const h4_double4 *v, const h4_forces *f, const double *t,
               const double *dt, double atime) {
    if (!h || !r || !v || !f || !t || !dt) return fail(H4_ERR_ARG, "h4_restore: null argument");
    if (!(atime >= 0.0) || !std::isfinite(atime)) return fail(H4_ERR_ARG, "h4_restore: bad atime");
    const size_t N = h->d.n;
    for (size_t i = 0; i < N; i++)
        if (!(dt[i] > 0.0) || !std::isfinite(t[i]) || !std::isfinite(dt[i]))
            return fail(H4_ERR_ARG, "h4_restore: bad t/dt at particle " + std::to_string(i));
    // masses rounded to float as in h4_create
    std::vector<h4_double4> rr(r, r + N);
    for (auto &p : rr) p.w = (double)(float)p.w;
    cudaStream_t s = h->stream;
    H4_TRY(cudaMemcpyAsync(h->d.r, rr.data(), N * 32, cudaMemcpyHostToDevice, s), "restore r");
    H4_TRY(cudaMemcpyAsync(h->d.v, v, N * 32, cudaMemcpyHostToDevice, s), "restore v");
    H4_TRY(cudaMemcpyAsync(h->d.f, f, N * 48, cudaMemcpyHostToDevice, s), "restore f");
    H4_TRY(cudaMemcpyAsync(h->d.t, t, N * 8, cudaMemcpyHostToDevice, s), "restore t");
    H4_TRY(cudaMemcpyAsync(h->d.dt, dt, N * 8, cudaMemcpyHostToDevice, s), "restore dt");
    launch_set_atime(h->d, atime, s);
    h->launches += 1;
    int st = check_launch("h4_restore");
    if (st) return st;
    H4_TRY(cudaStreamSynchronize(s), "h4_restore");
    h->forces_ready = true;
    return H4_OK;
}

int h4_download_predicted(h4_handle h, h4_double4 *pr, h4_double4 *pv) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    const size_t N = h->d.n;
    if (pr) H4_TRY(cudaMemcpyAsync(pr, h->d.pr, N * 32, cudaMemcpyDeviceToHost, h->stream), "download pr");
    if (pv) H4_TRY(cudaMemcpyAsync(pv, h->d.pv, N * 32, cudaMemcpyDeviceToHost, h->stream), "download pv");
    H4_TRY(cudaStreamSynchronize(h->stream), "download predicted");
    return H4_OK;
}

int h4_forces_for(h4_handle h, const h4_double4 *pr, const h4_double4 *pv, unsigned int nact,
                  const unsigned int *move, h4_forces *out) {
    if (!h || !pr || !pv || !move || !out) return fail(H4_ERR_ARG, "h4_forces_for: null argument");
    if (nact == 0) return H4_OK;
    if (nact > (unsigned)h->d.n) return fail(H4_ERR_ARG, "h4_forces_for: nact > n");
    for (unsigned k = 0; k < nact; k++)
        if (move[k] >= (unsigned)h->d.n) return fail(H4_ERR_ARG, "h4_forces_for: index out of range");
    const size_t N = h->d.n;
    cudaStream_t s = h->stream;
    H4_TRY(cudaMemcpyAsync(h->d.pr, pr, N * 32, cudaMemcpyHostToDevice, s), "h4_forces_for pr");
    H4_TRY(cudaMemcpyAsync(h->d.pv, pv, N * 32, cudaMemcpyHostToDevice, s), "h4_forces_for pv");
    H4_TRY(cudaMemcpyAsync(h->d.move, move, (size_t)nact * 4, cudaMemcpyHostToDevice, s), "h4_forces_for move");
    if (h->d.mixed) {   // the mixed kernels read the FP32 j data of these predictors
        launch_pack_j(h->d, s);
        h->launches += 1;
    }
    int st = set_nact(h, nact);
    if (st) return st;
    cudaEventRecord(h->ev0, s);
    launch_force(h, s, (long long)nact);
    cudaEventRecord(h->ev1, s);
    if ((st = check_launch("h4_forces_for"))) return st;
    if ((st = sync_ctrl(h))) return st;
    cudaEventElapsedTime(&h->last_force_ms, h->ev0, h->ev1);
    // Fixed-order reduction of the partial sums on the device, into a
    // temporary buffer (the handle's forces are left as they are).
    double *dout = nullptr;
    H4_TRY(cudaMallocAsync((void **)&dout, (size_t)nact * 6 * sizeof(double), s), "h4_forces_for buffer");
    launch_reduce_to(h->d, dout, s);
    h->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)nact * 6 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(dout, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "h4_forces_for");
    return H4_OK;
}

// Device positions and stream of a handle, for the diagnostics translation
// unit (not part of the public header).
int h4_internal_positions(h4_handle h, const void **r, int *n, void **stream) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    *r = h->d.r;
    *n = h->d.n;
    *stream = (void *)h->stream;
    return H4_OK;
}

int h4_last_timings(h4_handle h, float *force_ms, float *advance_ms) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    if (force_ms) {
        cudaError_t e = cudaEventSynchronize(h->ev1);
        if (e == cudaSuccess) cudaEventElapsedTime(&h->last_force_ms, h->ev0, h->ev1);
        *force_ms = h->last_force_ms;
    }
    if (advance_ms) *advance_ms = h->last_advance_ms;
    return H4_OK;
}

int h4_nact_histogram(h4_handle h, unsigned long long counts[32]) {
    if (!h || !counts) return fail(H4_ERR_ARG, "null argument");
    int st = sync_ctrl(h);
    if (st) return st;
    for (int k = 0; k < 32; k++) counts[k] = h->h_ctrl->nact_hist[k];
    return H4_OK;
}

int h4_phase_times(h4_handle h, double ms[H4_PHASES], unsigned long long counts[H4_PHASES]) {
    if (!h) return fail(H4_ERR_ARG, "null handle");
    for (int p = 0; p < PH_COUNT; p++) {
        phase_resolve(h->phase[p]);
        if (ms) ms[p] = h->phase[p].total_ms;
        if (counts) counts[p] = h->phase[p].count;
    }
    return H4_OK;
}

const char *h4_phase_name(int phase) {
    return (phase >= 0 && phase < PH_COUNT) ? kPhaseNames[phase] : "";
}

int h4_kernel_launches(h4_handle h, unsigned long long *count) {
    if (!h || !count) return fail(H4_ERR_ARG, "null argument");
    *count = h->launches;
    return H4_OK;
}

int h4_selftest_bounded_wait(double seconds, int *timed_out) {
    if (!(seconds > 0.0) || seconds > 5.0 || !timed_out)
        return fail(H4_ERR_ARG, "h4_selftest_bounded_wait: seconds in (0, 5], timed_out not NULL");
    cudaError_t e = selftest_bounded_wait(seconds, timed_out);
    if (e != cudaSuccess) return cuda_fail(e, "h4_selftest_bounded_wait");
    return H4_OK;
}

int h4_probe_peaks(double *fp64_flops, double *fp32_flops) {
    cudaError_t e = probe_peaks(fp64_flops, fp32_flops);
    if (e != cudaSuccess) return cuda_fail(e, "h4_probe_peaks");
    return H4_OK;
}

}  // extern "C"
