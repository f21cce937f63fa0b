// Tsit5 on the GPU for one network: `solve(ODEProblem(nw, u0, tspan, p), Tsit5())`
// (src/post_utils.jl:43-100 wraps the RHS; the stepper itself is OrdinaryDiffEqTsit5).
//
// The state, the stage vectors, the error norm and the step controller are FP64 on the
// device; the RHS runs in the handle's precision (an FP32 handle converts each stage
// state to FP32 and the stage derivative back).  Stage combinations use the operation
// order of the CPU oracle's Tsit5 (acc = Σ_j a_sj·k_j left to right, y = u + h·acc, no
// fused multiply-adds).  Step control stays on the device: the step size, the time and
// the accept flag live in device memory, so the host enqueues steps without waiting; one
// step is captured into a CUDA graph and replayed, and the host reads the status every
// few steps.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nd_internal.h"

namespace nd {

namespace {

constexpr int kSB = 256;

// Tsitouras (2011) 5(4) tableau; b equals the last row of a (FSAL), btilde = b - bhat.
__constant__ double c_a[7][6];
__constant__ double c_bt[7];

const double h_c[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
const double h_a[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
const double h_bt[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                        -0.1447110071732629,     0.5823571654525552,     -0.45808210592918697,
                        0.015151515151515152};

// Controller state in device memory.
struct Ctl {
    double t, t1, dt, qold, eest;
    double reltol, abstol;
    long long naccept, nreject, nsteps, max_steps;
    int done;    // 1 when t reached t1 (or a failure stopped the solve)
    int status;  // ND_OK, ND_ERR_MAXITERS, ND_ERR_NOT_CONVERGED (step size underflow)
    int accept;  // last step accepted
};

__global__ void stage_kernel(int s, int64_t n, const double* __restrict__ u, double* const* __restrict__ k,
                             double* __restrict__ y, const Ctl* ctl) {
    if (ctl->done) return;
    const double h = ctl->dt;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int j = 0; j < s; ++j) acc = __dadd_rn(acc, __dmul_rn(c_a[s][j], k[j][i]));
        y[i] = __dadd_rn(u[i], __dmul_rn(h, acc));
    }
}

__global__ void to_f32_kernel(int64_t n, const double* __restrict__ x, float* __restrict__ y, const Ctl* ctl) {
    if (ctl && ctl->done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}
__global__ void to_f64_kernel(int64_t n, const float* __restrict__ x, double* __restrict__ y, const Ctl* ctl) {
    if (ctl && ctl->done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (double)x[i];
}

// Per-block partial sums of ((h Σ btilde_j k_j) / (abstol + reltol max(|u|,|y|)))^2, fixed order.
__global__ void error_kernel(int64_t n, const double* __restrict__ u, const double* __restrict__ ynew,
                             double* const* __restrict__ k, double* __restrict__ partial, const Ctl* ctl) {
    __shared__ double red[kSB];
    double s = 0.0;
    if (!ctl->done) {
        const double h = ctl->dt;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            double acc = 0.0;
            for (int j = 0; j < 7; ++j) acc = __dadd_rn(acc, __dmul_rn(c_bt[j], k[j][i]));
            const double e = __dmul_rn(h, acc);
            const double sc = ctl->abstol + ctl->reltol * fmax(fabs(u[i]), fabs(ynew[i]));
            const double r = e / sc;
            s += r * r;
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = kSB / 2; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Step-size control (PI controller, the oracle's constants) on one thread.
__global__ void control_kernel(int nblocks, int64_t n, const double* __restrict__ partial, Ctl* ctl) {
    if (threadIdx.x != 0 || blockIdx.x != 0 || ctl->done) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partial[b];
    double EEst = sqrt(s / (double)(n > 0 ? n : 1));
    if (!(EEst == EEst)) EEst = 1e10;
    const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, gamma = 0.9, qmin = 0.2, qmax = 10.0;
    const double q11 = pow(EEst, beta1);
    ctl->eest = EEst;
    ctl->nsteps++;
    if (EEst <= 1.0) {
        double q = q11 / pow(ctl->qold, beta2);
        q = fmax(1.0 / qmax, fmin(1.0 / qmin, q / gamma));
        const double tn = ctl->t + ctl->dt;
        ctl->t = (fabs(ctl->t1 - tn) <= 1e-14 * fmax(1.0, fabs(ctl->t1))) ? ctl->t1 : tn;
        ctl->qold = fmax(EEst, 1e-4);
        ctl->naccept++;
        ctl->accept = 1;
        ctl->dt = ctl->dt / q;
    } else {
        ctl->nreject++;
        ctl->accept = 0;
        ctl->dt = ctl->dt / fmin(1.0 / qmin, q11 / gamma);
    }
    if (ctl->t >= ctl->t1) {
        ctl->done = 1;
        ctl->status = ND_OK;
    } else if (ctl->nsteps >= ctl->max_steps) {
        ctl->done = 1;
        ctl->status = ND_ERR_MAXITERS;
    } else if (ctl->dt < 1e-14 * fmax(1.0, fabs(ctl->t))) {
        ctl->done = 1;
        ctl->status = ND_ERR_NOT_CONVERGED;
    } else if (ctl->t1 - ctl->t < ctl->dt * (1 + 1e-12)) {
        ctl->dt = ctl->t1 - ctl->t;
    }
}

// Accepted step: u <- y (the 7th stage state), k1 <- k7 (FSAL).  `just` = the controller's
// accept flag of this step; runs even when the step ended the solve.
__global__ void accept_kernel(int64_t n, double* __restrict__ u, const double* __restrict__ y, double* __restrict__ k0,
                              const double* __restrict__ k6, const Ctl* ctl, int* last_seen) {
    if (!ctl->accept) return;
    if (ctl->done && *last_seen) return;  // step after completion: nothing to move
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        u[i] = y[i];
        k0[i] = k6[i];
    }
}
__global__ void mark_kernel(const Ctl* ctl, int* last_seen) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && ctl->done) *last_seen = 1;
}

struct Workspace {
    int64_t n = 0;
    double* k[7] = {};
    double* y = nullptr;
    double** kptr = nullptr;
    float* y32 = nullptr;
    float* k32 = nullptr;
    double* partial = nullptr;
    Ctl* ctl = nullptr;
    int* last_seen = nullptr;
    int nblocks = 0;
};

void free_ws(Workspace& w) {
    for (auto& p : w.k) cudaFree(p);
    cudaFree(w.y);
    cudaFree(w.kptr);
    cudaFree(w.y32);
    cudaFree(w.k32);
    cudaFree(w.partial);
    cudaFree(w.ctl);
    cudaFree(w.last_seen);
    w = Workspace{};
}

bool g_tableau_uploaded[64] = {};

}  // namespace

// RHS into an FP64 derivative from an FP64 state, in the handle's precision.
static int rhs_f64(nd_handle* h, Workspace& w, double* du, const double* y, const void* p, const Ctl* ctl,
                   cudaStream_t s) {
    const int64_t n = w.n;
    const unsigned g = (unsigned)std::min<int64_t>((n + kSB - 1) / kSB, 152 * 8);
    if (h->dtype == ND_F64) return nd_rhs(h, ND_F64, du, n, y, n, p, h->pdim, 0.0, s);
    to_f32_kernel<<<g, kSB, 0, s>>>(n, y, w.y32, ctl);
    int rc = nd_rhs(h, ND_F32, w.k32, n, w.y32, n, p, h->pdim, 0.0, s);
    if (rc != ND_OK) return rc;
    to_f64_kernel<<<g, kSB, 0, s>>>(n, w.k32, du, ctl);
    return ND_OK;
}

}  // namespace nd

using namespace nd;

extern "C" int nd_solve_tsit5(nd_handle* h, double* u, const void* p, double t0, double t1, double reltol,
                              double abstol, int64_t max_steps, nd_solve_stats* stats, void* stream) {
    clear_error();
    ND_NVTX("nd_solve_tsit5");
    if (!h || !u || !stats) return fail(ND_ERR_ARG, "nd_solve_tsit5: NULL argument");
    if (!(t1 > t0)) return fail(ND_ERR_ARG, "nd_solve_tsit5: t1 must be greater than t0");
    if (!(reltol > 0) || !(abstol > 0)) return fail(ND_ERR_ARG, "nd_solve_tsit5: tolerances must be positive");
    if (h->pdim > 0 && !p) return fail(ND_ERR_ARG, "nd_solve_tsit5: p is NULL");
    memset(stats, 0, sizeof *stats);
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !g_tableau_uploaded[dev]) {
        ND_CUDA_TRY(cudaMemcpyToSymbol(c_a, h_a, sizeof h_a));
        ND_CUDA_TRY(cudaMemcpyToSymbol(c_bt, h_bt, sizeof h_bt));
        g_tableau_uploaded[dev] = true;
    }
    cudaStream_t s;
    ND_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t ev;
    ND_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    // order after the caller's stream
    ND_CUDA_TRY(cudaEventRecord(ev, (cudaStream_t)stream));
    ND_CUDA_TRY(cudaStreamWaitEvent(s, ev, 0));

    Workspace w;
    w.n = h->dim;
    const int64_t n = w.n;
    w.nblocks = (int)std::min<int64_t>((n + kSB - 1) / kSB, 152 * 8);
    const unsigned g = (unsigned)w.nblocks;
    int rc = ND_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(s);
        free_ws(w);
        cudaEventDestroy(ev);
        cudaStreamDestroy(s);
    };
#define ND_WS(expr)                                      \
    do {                                                 \
        cudaError_t _e = (expr);                         \
        if (_e != cudaSuccess) {                         \
            rc = cuda_fail(_e, #expr);                   \
            cleanup();                                   \
            return rc;                                   \
        }                                                \
    } while (0)
    for (auto& k : w.k) ND_WS(cudaMalloc(&k, sizeof(double) * std::max<int64_t>(n, 1)));
    ND_WS(cudaMalloc(&w.y, sizeof(double) * std::max<int64_t>(n, 1)));
    ND_WS(cudaMalloc(&w.kptr, sizeof(double*) * 7));
    ND_WS(cudaMemcpy(w.kptr, w.k, sizeof(double*) * 7, cudaMemcpyHostToDevice));
    if (h->dtype == ND_F32) {
        ND_WS(cudaMalloc(&w.y32, sizeof(float) * std::max<int64_t>(n, 1)));
        ND_WS(cudaMalloc(&w.k32, sizeof(float) * std::max<int64_t>(n, 1)));
    }
    ND_WS(cudaMalloc(&w.partial, sizeof(double) * w.nblocks));
    ND_WS(cudaMalloc(&w.ctl, sizeof(Ctl)));
    ND_WS(cudaMalloc(&w.last_seen, sizeof(int)));
    ND_WS(cudaMemsetAsync(w.last_seen, 0, sizeof(int), s));

    // Initial step (Hairer & Wanner, order 5), on the host from two RHS evaluations.
    std::vector<double> hu(n), hk0(n), hk1(n);
    Ctl c{};
    c.t = t0;
    c.t1 = t1;
    c.reltol = reltol;
    c.abstol = abstol;
    c.qold = 1e-4;
    c.max_steps = max_steps > 0 ? max_steps : 1000000000ll;
    c.done = 0;
    c.status = ND_OK;
    ND_WS(cudaMemcpyAsync(w.ctl, &c, sizeof c, cudaMemcpyHostToDevice, s));
    if ((rc = rhs_f64(h, w, w.k[0], u, p, nullptr, s)) != ND_OK) {
        cleanup();
        return rc;
    }
    ND_WS(cudaMemcpyAsync(hu.data(), u, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    ND_WS(cudaMemcpyAsync(hk0.data(), w.k[0], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    ND_WS(cudaStreamSynchronize(s));
    double d0 = 0, d1 = 0;
    for (int64_t i = 0; i < n; ++i) {
        const double sc = abstol + fabs(hu[i]) * reltol;
        d0 += (hu[i] / sc) * (hu[i] / sc);
        d1 += (hk0[i] / sc) * (hk0[i] / sc);
    }
    d0 = sqrt(d0 / (double)(n ? n : 1));
    d1 = sqrt(d1 / (double)(n ? n : 1));
    double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
    h0 = fmin(h0, t1 - t0);
    std::vector<double> hy(n);
    for (int64_t i = 0; i < n; ++i) hy[i] = hu[i] + h0 * hk0[i];
    ND_WS(cudaMemcpyAsync(w.y, hy.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    if ((rc = rhs_f64(h, w, w.k[1], w.y, p, nullptr, s)) != ND_OK) {
        cleanup();
        return rc;
    }
    ND_WS(cudaMemcpyAsync(hk1.data(), w.k[1], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    ND_WS(cudaStreamSynchronize(s));
    double d2 = 0;
    for (int64_t i = 0; i < n; ++i) {
        const double sc = abstol + fabs(hu[i]) * reltol;
        const double r = (hk1[i] - hk0[i]) / sc;
        d2 += r * r;
    }
    d2 = sqrt(d2 / (double)(n ? n : 1)) / h0;
    const double h1 = (fmax(d1, d2) <= 1e-15) ? fmax(1e-6, h0 * 1e-3) : pow(0.01 / fmax(d1, d2), 1.0 / 5.0);
    c.dt = fmin(fmin(100 * h0, h1), t1 - t0);
    ND_WS(cudaMemcpyAsync(w.ctl, &c, sizeof c, cudaMemcpyHostToDevice, s));
    stats->nf = 2;

    // One step, captured into a graph: stages 2..7 (k1 is valid: initial RHS / FSAL),
    // error norm, controller, accept.
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ND_WS(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    bool ok = true;
    for (int st = 1; st < 7 && ok; ++st) {
        stage_kernel<<<g, kSB, 0, s>>>(st, n, u, w.kptr, w.y, w.ctl);
        ok = rhs_f64(h, w, w.k[st], w.y, p, w.ctl, s) == ND_OK;
    }
    error_kernel<<<g, kSB, 0, s>>>(n, u, w.y, w.kptr, w.partial, w.ctl);
    mark_kernel<<<1, 32, 0, s>>>(w.ctl, w.last_seen);
    control_kernel<<<1, 32, 0, s>>>(w.nblocks, n, w.partial, w.ctl);
    accept_kernel<<<g, kSB, 0, s>>>(n, u, w.y, w.k[0], w.k[6], w.ctl, w.last_seen);
    cudaError_t cap = cudaStreamEndCapture(s, &graph);
    if (!ok) {
        if (graph) cudaGraphDestroy(graph);
        rc = ND_ERR_CUDA;
        cleanup();
        return rc;
    }
    ND_WS(cap);
    ND_WS(cudaGraphInstantiate(&exec, graph, 0));
    const int kBatch = 16;
    for (;;) {
        for (int i = 0; i < kBatch; ++i) ND_WS(cudaGraphLaunch(exec, s));
        ND_WS(cudaMemcpyAsync(&c, w.ctl, sizeof c, cudaMemcpyDeviceToHost, s));
        ND_WS(cudaStreamSynchronize(s));
        if (c.done) break;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    stats->naccept = c.naccept;
    stats->nreject = c.nreject;
    stats->nf += 6 * (c.naccept + c.nreject);
    stats->t_final = c.t;
    stats->dt_last = c.dt;
    stats->status = c.status;
    // order the caller's stream after the solve
    ND_WS(cudaEventRecord(ev, s));
    ND_WS(cudaStreamWaitEvent((cudaStream_t)stream, ev, 0));
    cleanup();
#undef ND_WS
    if (c.status != ND_OK)
        return fail(c.status, c.status == ND_ERR_MAXITERS ? "nd_solve_tsit5: maximum number of steps reached"
                                                          : "nd_solve_tsit5: step size underflow");
    return ND_OK;
}
