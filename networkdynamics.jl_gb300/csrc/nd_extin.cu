// External inputs and loopback edges: the two device copies the reference's core loop
// makes for them, as entry points a host that keeps its own components can call.
//
//   nd_collect_externals  extbuf[k] = u[idx[k]] (a state) or o[idx[k]] (an output), the
//                         ExtMap gather of src/external_inputs.jl:51-80 (collect_ext_kernel!)
//                         that fills the external-input buffer before the components run;
//   nd_apply_loopback     aggbuf[agg[k]] = obuf[out[k]], the copy of an injector's
//                         output into its satellite's aggregated input
//                         (src/post_utils.jl:213-248, applied at src/coreloop.jl:47).
//
// No library component reads external inputs or is an injector with a feed-forward
// output, so nd_rhs never needs them; networks that would are rejected at construction.
// One thread per entry, grid-stride; the indices are 0-based and must lie inside the
// buffers (the caller's map, as the reference builds it).
#include <algorithm>

#include "nd_internal.h"

namespace nd {

namespace {

template <typename T>
__global__ void collect_kernel(int64_t n, const int64_t* __restrict__ idx, const uint8_t* __restrict__ from_state,
                               T* __restrict__ ext, const T* __restrict__ u, const T* __restrict__ o) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx[k];
        ext[k] = from_state[k] ? u[i] : o[i];
    }
}

template <typename T>
__global__ void loopback_kernel(int64_t n, const int64_t* __restrict__ out_idx, const int64_t* __restrict__ agg_idx,
                                T* __restrict__ agg, const T* __restrict__ obuf) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        agg[agg_idx[k]] = obuf[out_idx[k]];
}

unsigned grid_for_n(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

}  // namespace

}  // namespace nd

using namespace nd;

extern "C" int nd_collect_externals(int dtype, int64_t n, const int64_t* idx, const uint8_t* from_state, void* extbuf,
                                    const void* u, const void* o, void* stream) {
    clear_error();
    ND_NVTX("nd_collect_externals");
    if (dtype != ND_F32 && dtype != ND_F64) return fail(ND_ERR_DTYPE, "nd_collect_externals: dtype must be ND_F32 or ND_F64");
    if (n < 0) return fail(ND_ERR_ARG, "nd_collect_externals: negative length");
    if (n == 0) return ND_OK;
    if (!idx || !from_state || !extbuf) return fail(ND_ERR_ARG, "nd_collect_externals: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == ND_F64)
        collect_kernel<double><<<grid_for_n(n), 256, 0, s>>>(n, idx, from_state, static_cast<double*>(extbuf),
                                                             static_cast<const double*>(u), static_cast<const double*>(o));
    else
        collect_kernel<float><<<grid_for_n(n), 256, 0, s>>>(n, idx, from_state, static_cast<float*>(extbuf),
                                                            static_cast<const float*>(u), static_cast<const float*>(o));
    const cudaError_t err = cudaGetLastError();
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_collect_externals");
}

extern "C" int nd_apply_loopback(int dtype, int64_t n, const int64_t* out_idx, const int64_t* agg_idx, void* aggbuf,
                                 const void* obuf, void* stream) {
    clear_error();
    ND_NVTX("nd_apply_loopback");
    if (dtype != ND_F32 && dtype != ND_F64) return fail(ND_ERR_DTYPE, "nd_apply_loopback: dtype must be ND_F32 or ND_F64");
    if (n < 0) return fail(ND_ERR_ARG, "nd_apply_loopback: negative length");
    if (n == 0) return ND_OK;
    if (!out_idx || !agg_idx || !aggbuf || !obuf) return fail(ND_ERR_ARG, "nd_apply_loopback: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == ND_F64)
        loopback_kernel<double><<<grid_for_n(n), 256, 0, s>>>(n, out_idx, agg_idx, static_cast<double*>(aggbuf),
                                                              static_cast<const double*>(obuf));
    else
        loopback_kernel<float><<<grid_for_n(n), 256, 0, s>>>(n, out_idx, agg_idx, static_cast<float*>(aggbuf),
                                                             static_cast<const float*>(obuf));
    const cudaError_t err = cudaGetLastError();
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_apply_loopback");
}
