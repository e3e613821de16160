// mathcheck.cu -- pbsm3d_math_eval: the library's table-driven FP64 routines
// (fp64_math.cuh) and CUDA's own functions evaluated side by side on the
// device, so their agreement can be measured directly (ulp bounds, special
// values) rather than only through the assembly's results.
#include <string>

#include "fp64_math.cuh"
#include "pbsm3d_internal.cuh"

namespace pbsm {
namespace {

__device__ MathTables g_mc_tables;

__global__ void k_math_eval(int fn, int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                            double* __restrict__ out) {
    __shared__ MathTables t;
    math_tables_load(t, &g_mc_tables);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = a[i];
        const double y = b ? b[i] : 0.0;
        double r;
        switch (fn) {
            case PBSM3D_MATH_EXP: r = exp_t(x, t); break;
            case PBSM3D_MATH_LOG: r = log_t(x, t); break;
            case PBSM3D_MATH_RCP: r = rcp_t(x); break;
            case PBSM3D_MATH_DIV: r = div_t(x, y); break;
            case PBSM3D_MATH_POW: r = pow_t(x, y, t); break;
            case PBSM3D_MATH_F32: r = (double)f32_rn(x); break;
            case PBSM3D_MATH_CUDA_EXP: r = exp(x); break;
            case PBSM3D_MATH_CUDA_LOG: r = log(x); break;
            case PBSM3D_MATH_CUDA_RCP: r = 1.0 / x; break;
            case PBSM3D_MATH_CUDA_DIV: r = x / y; break;
            case PBSM3D_MATH_CUDA_POW: r = pow(x, y); break;
            default: r = (double)(float)x; break;  // PBSM3D_MATH_CUDA_F32
        }
        out[i] = r;
    }
}

__device__ double g_fp64_sink;

// FP64 issue rate: every thread runs eight independent FMA chains (no
// memory traffic), so the FP64 pipe is the only limit.  The chains contract
// towards a fixed point (a < 1), so the values stay normal.
__global__ void __launch_bounds__(256) k_fp64_rate(int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == -1.0) g_fp64_sink = s;  // never true; keeps the chains
}

}  // namespace
}  // namespace pbsm

using namespace pbsm;

extern "C" int pbsm3d_fp64_rate(double* fma_per_s) {
    if (!fma_per_s) {
        set_global_error("pbsm3d_fp64_rate: invalid argument");
        return PBSM3D_ERR_INVALID_ARG;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    // two resident waves of 256-thread blocks a SM; warm-up launches let the
    // clocks settle, then the best of three
    const int grid = 8 * sms, iters = 4096;
    float best = 0.f;
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {  // ~0.1 s of load: the clocks settle
        k_fp64_rate<<<grid, 256>>>(iters, 0.999999, 1e-6);
        e = cudaGetLastError();
    }
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
        float ms = 0.f;
        cudaEventRecord(ev[0]);
        k_fp64_rate<<<grid, 256>>>(iters, 0.999999, 1e-6);
        cudaEventRecord(ev[1]);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        if (e == cudaSuccess && ms > 0.f && (best == 0.f || ms < best)) best = ms;
    }
    for (auto& x : ev)
        if (x) cudaEventDestroy(x);
    if (e != cudaSuccess || !(best > 0.f)) {
        set_global_error(std::string("pbsm3d_fp64_rate: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "no time"));
        return PBSM3D_ERR_CUDA;
    }
    *fma_per_s = (double)grid * 256 * iters * 8 / (best * 1e-3);
    return PBSM3D_OK;
}

extern "C" int pbsm3d_math_eval(int32_t fn, int64_t n, const double* a, const double* b, double* out) {
    if (n < 0 || (n > 0 && (!a || !out)) || fn < PBSM3D_MATH_EXP || fn > PBSM3D_MATH_CUDA_F32 ||
        ((fn == PBSM3D_MATH_DIV || fn == PBSM3D_MATH_POW || fn == PBSM3D_MATH_CUDA_DIV ||
          fn == PBSM3D_MATH_CUDA_POW) && n > 0 && !b)) {
        set_global_error("pbsm3d_math_eval: invalid argument");
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (n == 0) return PBSM3D_OK;
    MathTables h;
    math_tables_fill(h);
    cudaError_t e = cudaMemcpyToSymbol(g_mc_tables, &h, sizeof(h));
    if (e == cudaSuccess) {
        const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
        k_math_eval<<<grid, 256>>>(fn, n, a, b, out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        set_global_error(std::string("pbsm3d_math_eval: ") + cudaGetErrorString(e));
        return PBSM3D_ERR_CUDA;
    }
    return PBSM3D_OK;
}
