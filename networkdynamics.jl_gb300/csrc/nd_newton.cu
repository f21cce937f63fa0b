// Steady states of any network of the library: Newton's method with
// restarted GMRES on the assembled sparse Jacobian, the GPU counterpart of
// find_fixpoint(nw, x0, p) (src/initialization.jl:44-144), which solves a
// SteadyStateProblem with NonlinearSolve's Newton-type root finders.
//
//   F(u) = nw(du, u, p, t); stop when max|F| <= tol (the reference's residual norm,
//   src/initialization.jl:129).  Before the first step the RHS is checked for NaN, as the
//   reference does (:75-126).
//   Newton step: J δ = -F with J = ∂F/∂u at u (nd_jacobian), solved by GMRES(m), right-
//   preconditioned by the Jacobian's diagonal (Jacobi), with Arnoldi by classical
//   Gram-Schmidt applied twice and Givens rotations, to a relative residual
//   η = min(1e-2, max|F|), at most `max_restarts` cycles; then a backtracking line search
//   on max|F| (λ = 1, 1/2, ... 2^-10).  Singular Jacobians with a consistent right-hand
//   side (the phase shift of Kuramoto / swing networks) are fine for GMRES started from 0.
//
// Vector work runs in small kernels: CSR products, and dot products reduced in two
// deterministic passes (block partials, then one block), so a solve repeats bit for bit.
// The Hessenberg least-squares problem (at most m + 1 rows) lives on the host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "nd_internal.h"

namespace nd {

namespace {

constexpr int kNB = 256;        // threads per block of the vector kernels
constexpr int kDotBlocks = 304; // partial sums per dot product (2 per SM)
constexpr int kMaxKrylov = 64;

__global__ void spmv_kernel(int64_t n, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                            const double* __restrict__ val, const double* __restrict__ x, double* __restrict__ y) {
    for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB) {
        double s = 0.0;
        for (int32_t k = __ldg(rowptr + i); k < __ldg(rowptr + i + 1); ++k)
            s = __dadd_rn(s, __dmul_rn(__ldg(val + k), __ldg(x + __ldg(col + k))));
        y[i] = s;
    }
}

// partial[b * nv + j] = sum over this block's slice of V[j] . w, for j < nv
__global__ void multidot_partial(int64_t n, int nv, const double* __restrict__ V, int64_t ldv,
                                 const double* __restrict__ w, double* __restrict__ partial) {
    __shared__ double red[kNB / 32];
    for (int j = 0; j < nv; ++j) {
        double s = 0.0;
        for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB)
            s = __dadd_rn(s, __dmul_rn(V[j * ldv + i], w[i]));
        for (int off = 16; off > 0; off >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, off));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int k = 0; k < kNB / 32; ++k) t = __dadd_rn(t, red[k]);
            partial[(int64_t)blockIdx.x * nv + j] = t;
        }
        __syncthreads();
    }
}

// out[j] = sum over blocks of partial[b * nv + j]
__global__ void multidot_final(int nblocks, int nv, const double* __restrict__ partial, double* __restrict__ out) {
    const int j = threadIdx.x;
    if (j >= nv) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; ++b) t = __dadd_rn(t, partial[(int64_t)b * nv + j]);
    out[j] = t;
}

// max |x| per block, then over blocks (deterministic)
__global__ void absmax_partial(int64_t n, const double* __restrict__ x, double* __restrict__ partial,
                               int* __restrict__ nan_flag) {
    __shared__ double red[kNB / 32];
    double m = 0.0;
    bool nan = false;
    for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB) {
        const double v = x[i];
        nan |= v != v;
        m = fmax(m, fabs(v));
    }
    if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(nan_flag, 1);
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kNB / 32; ++k) t = fmax(t, red[k]);
        partial[blockIdx.x] = t;
    }
}

__global__ void absmax_final(int nblocks, const double* __restrict__ partial, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; ++b) t = fmax(t, partial[b]);
    out[0] = t;
}

// y = a * x + b * y with scalars from the host
__global__ void axpby_kernel(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB)
        y[i] = __dadd_rn(__dmul_rn(a, x[i]), __dmul_rn(b, y[i]));
}

// w -= sum_j h[j] V[j]  (h on the device, j < nv)
__global__ void orth_update(int64_t n, int nv, const double* __restrict__ V, int64_t ldv, const double* __restrict__ h,
                            double* __restrict__ w) {
    for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB) {
        double s = w[i];
        for (int j = 0; j < nv; ++j) s = __dsub_rn(s, __dmul_rn(h[j], V[j * ldv + i]));
        w[i] = s;
    }
}

// x += sum_j c[j] V[j]
__global__ void combine_kernel(int64_t n, int nv, const double* __restrict__ V, int64_t ldv, const double* __restrict__ c,
                               double* __restrict__ x) {
    for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB) {
        double s = x[i];
        for (int j = 0; j < nv; ++j) s = __dadd_rn(s, __dmul_rn(c[j], V[j * ldv + i]));
        x[i] = s;
    }
}

// dinv[i] = 1 / J[i][i] (1 where the diagonal is zero or absent): the Jacobi scaling
__global__ void diag_inverse_kernel(int64_t n, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                    const double* __restrict__ val, double* __restrict__ dinv) {
    for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB) {
        double d = 0.0;
        for (int32_t k = __ldg(rowptr + i); k < __ldg(rowptr + i + 1); ++k)
            if (__ldg(col + k) == (int32_t)i) d = __ldg(val + k);
        dinv[i] = d != 0.0 && d == d ? __ddiv_rn(1.0, d) : 1.0;
    }
}

// z = dinv * x (elementwise)
__global__ void scale_kernel(int64_t n, const double* __restrict__ dinv, const double* __restrict__ x,
                             double* __restrict__ z) {
    for (int64_t i = (int64_t)blockIdx.x * kNB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNB)
        z[i] = __dmul_rn(dinv[i], x[i]);
}

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + kNB - 1) / kNB, 152 * 8)); }

struct Workspace {
    double* buf = nullptr;
    ~Workspace() { cudaFree(buf); }
};

}  // namespace

size_t GmresSolver::doubles(int64_t n, int m) { return (size_t)n * (3 + m + 1) + (size_t)kDotBlocks * (m + 1) + 2 * (kMaxKrylov + 2); }

void GmresSolver::attach(double* buf, int64_t n_, int m_, cudaStream_t s_) {
    n = n_;
    m = std::max(2, std::min(m_, kMaxKrylov));
    s = s_;
    w = buf;
    dinv = w + n;
    z = dinv + n;
    V = z + n;
    partial = V + (size_t)n * (m + 1);
    dscal = partial + (size_t)kDotBlocks * (m + 1);
}

int GmresSolver::sync(const char* what) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? ND_OK : cuda_fail(e, what);
}

int GmresSolver::multidot(const double* Vb, int nv, const double* x, double* dots) {
    multidot_partial<<<kDotBlocks, kNB, 0, s>>>(n, nv, Vb, n, x, partial);
    multidot_final<<<1, 64, 0, s>>>(kDotBlocks, nv, partial, dscal);
    cudaMemcpyAsync(dots, dscal, nv * sizeof(double), cudaMemcpyDeviceToHost, s);
    return sync("gmres: dot");
}

void GmresSolver::jacobi(const int32_t* rowptr, const int32_t* col, const double* vals) {
    diag_inverse_kernel<<<grid_for(n), kNB, 0, s>>>(n, rowptr, col, vals, dinv);
}

// Restarted GMRES(m) for A x = b, x updated in place, right-preconditioned by the Jacobi
// scaling set by jacobi(); Arnoldi by classical Gram-Schmidt applied twice, Givens
// rotations on the host; stops at ||b - A x|| <= rtol ||b||.
int GmresSolver::solve(const int32_t* rowptr, const int32_t* col, const double* vals, const double* b, double* x,
                       double rtol, int restarts, double* rel_res) {
    const unsigned G = grid_for(n);
    const int64_t ldv = n;
    int rc;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m), dots(m + 1);
    double bnorm2 = 0.0;
    if ((rc = multidot(b, 1, b, &bnorm2)) != ND_OK) return rc;
    const double bnorm = std::sqrt(bnorm2);
    double res = 0.0;
    for (int cycle = 0; cycle < restarts; ++cycle) {
        // r = b - A x  (in V[0])
        spmv_kernel<<<G, kNB, 0, s>>>(n, rowptr, col, vals, x, V);
        axpby_kernel<<<G, kNB, 0, s>>>(n, 1.0, b, -1.0, V);
        double beta2 = 0.0;
        if ((rc = multidot(V, 1, V, &beta2)) != ND_OK) return rc;
        const double beta = std::sqrt(beta2);
        res = beta;
        if (beta <= rtol * bnorm || beta == 0.0) break;
        axpby_kernel<<<G, kNB, 0, s>>>(n, 0.0, V, 1.0 / beta, V);
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        for (; k < m; ++k) {
            double* vk1 = V + (size_t)(k + 1) * ldv;
            // right preconditioning: w = A D^-1 v_k
            scale_kernel<<<G, kNB, 0, s>>>(n, dinv, V + (size_t)k * ldv, z);
            spmv_kernel<<<G, kNB, 0, s>>>(n, rowptr, col, vals, z, vk1);
            for (int pass = 0; pass < 2; ++pass) {
                if ((rc = multidot(V, k + 1, vk1, dots.data())) != ND_OK) return rc;
                cudaMemcpyAsync(dscal, dots.data(), (k + 1) * sizeof(double), cudaMemcpyHostToDevice, s);
                orth_update<<<G, kNB, 0, s>>>(n, k + 1, V, ldv, dscal, vk1);
                for (int j = 0; j <= k; ++j) H[(size_t)j * m + k] = (pass ? H[(size_t)j * m + k] : 0.0) + dots[j];
            }
            double hn2 = 0.0;
            if ((rc = multidot(vk1, 1, vk1, &hn2)) != ND_OK) return rc;
            const double hn = std::sqrt(hn2);
            H[(size_t)(k + 1) * m + k] = hn;
            if (hn > 0) axpby_kernel<<<G, kNB, 0, s>>>(n, 0.0, vk1, 1.0 / hn, vk1);
            for (int j = 0; j < k; ++j) {
                const double a = H[(size_t)j * m + k], bb = H[(size_t)(j + 1) * m + k];
                H[(size_t)j * m + k] = cs[j] * a + sn[j] * bb;
                H[(size_t)(j + 1) * m + k] = -sn[j] * a + cs[j] * bb;
            }
            const double a = H[(size_t)k * m + k], bb = H[(size_t)(k + 1) * m + k];
            const double r = std::hypot(a, bb);
            cs[k] = r > 0 ? a / r : 1.0;
            sn[k] = r > 0 ? bb / r : 0.0;
            H[(size_t)k * m + k] = r;
            H[(size_t)(k + 1) * m + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            res = std::fabs(g[k + 1]);
            if (res <= rtol * bnorm || hn == 0.0) {
                ++k;
                break;
            }
        }
        for (int i = k - 1; i >= 0; --i) {
            double sacc = g[i];
            for (int j = i + 1; j < k; ++j) sacc -= H[(size_t)i * m + j] * y[j];
            const double d = H[(size_t)i * m + i];
            y[i] = d != 0.0 ? sacc / d : 0.0;
        }
        // x += D^-1 V y
        cudaMemcpyAsync(dscal, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(z, 0, n * sizeof(double), s);
        combine_kernel<<<G, kNB, 0, s>>>(n, k, V, ldv, dscal, z);
        scale_kernel<<<G, kNB, 0, s>>>(n, dinv, z, z);
        axpby_kernel<<<G, kNB, 0, s>>>(n, 1.0, z, 1.0, x);
        if ((rc = sync("gmres")) != ND_OK) return rc;
        if (res <= rtol * bnorm) break;
    }
    if (rel_res) *rel_res = bnorm > 0 ? res / bnorm : 0.0;
    return ND_OK;
}

void vec_axpby(int64_t n, double a, const double* x, double b, double* y, cudaStream_t s) {
    axpby_kernel<<<grid_for(n), kNB, 0, s>>>(n, a, x, b, y);
}

}  // namespace nd

using namespace nd;

extern "C" int nd_find_fixpoint(nd_handle* h, double* u, const double* p, double t, double tol, int max_newton,
                                int krylov_dim, int max_restarts, int32_t* iters, double* resid, void* stream) {
    clear_error();
    ND_NVTX("nd_find_fixpoint");
    if (!h || !u || !iters || !resid) return fail(ND_ERR_ARG, "nd_find_fixpoint: NULL argument");
    if (h->dtype != ND_F64) return fail(ND_ERR_DTYPE, "nd_find_fixpoint: FP64 handles only");
    if (h->pdim > 0 && !p) return fail(ND_ERR_ARG, "nd_find_fixpoint: p is NULL");
    if (!(tol > 0) || max_newton < 1) return fail(ND_ERR_ARG, "nd_find_fixpoint: tol must be > 0, max_newton >= 1");
    const int m = std::max(2, std::min(krylov_dim <= 0 ? 40 : krylov_dim, kMaxKrylov));
    const int restarts = max_restarts <= 0 ? 20 : max_restarts;
    *iters = 0;
    *resid = NAN;
    cudaStream_t s = (cudaStream_t)stream;
    int64_t nnz = 0;
    int rc = nd_jacobian_pattern(h, &nnz, nullptr, nullptr);
    if (rc != ND_OK) return rc;
    const int64_t n = h->dim;
    const JacPlan& J = h->jac;
    // device workspace: F, Fnew, trial u, δ, -F, the Jacobian values, the GMRES workspace
    // (w, D^-1, z, Krylov basis V[m+1][n], dot partials, scalars), the NaN flag
    const size_t doubles = (size_t)n * 5 + (size_t)std::max<int64_t>(nnz, 1) + GmresSolver::doubles(n, m);
    Workspace ws;
    cudaError_t err = cudaMalloc(&ws.buf, doubles * sizeof(double) + 64);
    if (err != cudaSuccess) return cuda_fail(err, "nd_find_fixpoint: workspace");
    double* F = ws.buf;
    double* Fn = F + n;
    double* ut = Fn + n;
    double* dlt = ut + n;
    double* negF = dlt + n;
    double* vals = negF + n;
    GmresSolver gm;
    gm.attach(vals + std::max<int64_t>(nnz, 1), n, m, s);
    int* nan_flag = reinterpret_cast<int*>(gm.dscal + 2 * (kMaxKrylov + 2));
    const unsigned G = grid_for(n);

    auto sync_err = [&](const char* what) -> int {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = cudaGetLastError();
        return e == cudaSuccess ? ND_OK : cuda_fail(e, what);
    };
    auto rhs = [&](double* out, const double* x) { return nd_rhs(h, ND_F64, out, n, x, n, p, h->pdim, t, s); };
    // max |x| and a NaN flag, on the host
    auto absmax = [&](const double* x, double* val, bool* nan) -> int {
        cudaMemsetAsync(nan_flag, 0, sizeof(int), s);
        absmax_partial<<<kDotBlocks, kNB, 0, s>>>(n, x, gm.partial, nan_flag);
        absmax_final<<<1, 32, 0, s>>>(kDotBlocks, gm.partial, gm.dscal);
        int flag = 0;
        cudaMemcpyAsync(val, gm.dscal, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&flag, nan_flag, sizeof(int), cudaMemcpyDeviceToHost, s);
        const int r = sync_err("nd_find_fixpoint: norm");
        *nan = flag != 0;
        return r;
    };

    if ((rc = rhs(F, u)) != ND_OK) return rc;
    double fmax = 0.0;
    bool nan = false;
    if ((rc = absmax(F, &fmax, &nan)) != ND_OK) return rc;
    if (nan || !(fmax == fmax)) {
        *resid = NAN;
        return fail(ND_ERR_NOT_CONVERGED, "Evaluation of network rhs resulted in NaNs (check u and p for NaN)");
    }
    int it = 0;
    while (fmax > tol && it < max_newton) {
        ++it;
        // Jacobian at u, then GMRES for J δ = -F from δ = 0
        if ((rc = nd_jacobian(h, ND_F64, vals, u, p, t, s)) != ND_OK) return rc;
        gm.jacobi(J.rowptr, J.colidx, vals);
        cudaMemsetAsync(dlt, 0, n * sizeof(double), s);
        cudaMemsetAsync(negF, 0, n * sizeof(double), s);  // 0 * (uninitialised) could be NaN
        axpby_kernel<<<G, kNB, 0, s>>>(n, -1.0, F, 0.0, negF);
        if ((rc = gm.solve(J.rowptr, J.colidx, vals, negF, dlt, std::min(1e-2, fmax), restarts, nullptr)) != ND_OK)
            return rc;
        // backtracking line search on max|F|
        double lam = 1.0, fnew = 0.0;
        bool accepted = false;
        for (int ls = 0; ls <= 10; ++ls, lam *= 0.5) {
            cudaMemcpyAsync(ut, u, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
            axpby_kernel<<<G, kNB, 0, s>>>(n, lam, dlt, 1.0, ut);
            if ((rc = rhs(Fn, ut)) != ND_OK) return rc;
            if ((rc = absmax(Fn, &fnew, &nan)) != ND_OK) return rc;
            if (!nan && fnew < fmax) {
                accepted = true;
                break;
            }
        }
        if (!accepted) break;  // no decrease along the Newton direction
        cudaMemcpyAsync(u, ut, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(F, Fn, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
        fmax = fnew;
    }
    if ((rc = sync_err("nd_find_fixpoint")) != ND_OK) return rc;
    *iters = it;
    *resid = fmax;
    if (!(fmax <= tol)) {
        char buf[200];
        snprintf(buf, sizeof buf, "Could not find fixpoint: residual %.3e after %d Newton iterations (tol %.1e)", fmax,
                 it, tol);
        return fail(ND_ERR_NOT_CONVERGED, buf);
    }
    return ND_OK;
}
