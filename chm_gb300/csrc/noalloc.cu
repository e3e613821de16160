// noalloc.cu -- pbsm3d_deposition_solve_noalloc: the deposition solve for
// callers that must not allocate device memory.
//
// Some hosts of this library own all device memory themselves: a model that
// reserves the GPU's memory when it starts and forbids allocation inside its
// time loop, or a framework whose memory pool is the only allocator allowed
// on the device.  They cannot use pbsm3d_create, which allocates the context.
// This entry point runs the Jacobi-preconditioned CG of the deposition
// system on arrays the caller passes in, and takes its work space (four
// vectors, the per-block partial sums and the solver scalars) from one
// file-scope __device__ array instead of cudaMalloc.  The array is sized for
// kNoAllocMaxFaces faces and lives on every device that loads the library
// until the process exits.
//
// Its address is looked up with cudaGetSymbolAddress once per device, by the
// first call made with that device current, and cached; make that first call
// before any stream capture.  The cache remembers the device context it was
// taken in (cuCtxGetId, reached through cudaGetDriverEntryPointByVersion, so
// the library needs no link to the driver library): after a cudaDeviceReset
// the next call looks the address up again in the new context.  Where the
// driver has no context ids the address is kept for the process, and the
// device must not be reset after the first call.  All calls share the one
// array: calls that overlap on a device (other host threads, other streams)
// race on it.  Each call clears the part that must start at zero (the
// reduction counters).
#include <cuda.h>
#include <math.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "pbsm3d_internal.cuh"

namespace pbsm {
namespace {

constexpr int64_t kNoAllocMaxFaces = 1 << 20;  // 1,048,576 faces: 32 MiB of vectors
constexpr int kNaMaxBlocks = 1216;
constexpr size_t kNaHeader = 65536;  // scalars + partials, 256-byte aligned offsets
constexpr size_t kNaBytes = kNaHeader + 4 * (size_t)kNoAllocMaxFaces * sizeof(double);
static_assert(sizeof(Scalars) + 4 * kNaMaxBlocks * sizeof(double) + 256 <= kNaHeader, "header too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct NaView {
    Scalars* sc;
    double* partials;
    double *r, *z, *p, *q;
};

NaView view_of(unsigned char* base) {
    NaView v;
    v.sc = reinterpret_cast<Scalars*>(base);
    v.partials = reinterpret_cast<double*>(base + 256);
    double* vec = reinterpret_cast<double*>(base + kNaHeader);
    v.r = vec;
    v.z = vec + kNoAllocMaxFaces;
    v.p = vec + 2 * kNoAllocMaxFaces;
    v.q = vec + 3 * kNoAllocMaxFaces;
    return v;
}

struct DepIn {
    int64_t n;
    const int32_t* nbr;  // [3][n]
    const double* diag;  // [n]
    const double* off;   // [3][n]
    const double* rhs;   // [n]
    double* x;           // [n]
};

__device__ __forceinline__ double apply_row(const DepIn& D, const double* v, int64_t i) {
    double a = D.diag[i] * v[i];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int32_t nb = D.nbr[j * D.n + i];
        if (nb >= 0) a += D.off[j * D.n + i] * v[nb];
    }
    return a;
}

// r = b, z = b / diag, p = z, x = 0; then (r, z), (b, b)
__global__ void __launch_bounds__(kBlock) k_na_init(DepIn D, NaView W, double tol, int maxit) {
    double acc[2] = {0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.n; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = D.rhs[i];
        const double zi = bi / D.diag[i];
        W.r[i] = bi;
        W.z[i] = zi;
        W.p[i] = zi;
        D.x[i] = 0.0;
        acc[0] += bi * zi;
        acc[1] += bi * bi;
    }
    double tot[2];
    if (block_partials_last<2>(acc, W.partials, &W.sc->counter[0], tot) && threadIdx.x == 0) {
        W.sc->rho = tot[0];
        W.sc->bnorm2 = tot[1];
        W.sc->rnorm2 = tot[1];
        W.sc->target2 = tol * tol * tot[1];
        W.sc->iter = 0;
        W.sc->maxit = maxit;
        W.sc->done = tot[1] == 0.0 ? 1 : 0;
    }
}

// q = A p; alpha = rho / (p, q)
__global__ void __launch_bounds__(kBlock) k_na_q(DepIn D, NaView W) {
    if (W.sc->done) return;
    double acc[1] = {0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.n; i += (int64_t)gridDim.x * blockDim.x) {
        const double qi = apply_row(D, W.p, i);
        W.q[i] = qi;
        acc[0] += W.p[i] * qi;
    }
    double tot[1];
    if (block_partials_last<1>(acc, W.partials, &W.sc->counter[0], tot) && threadIdx.x == 0) {
        if (!(tot[0] > 0.0))
            W.sc->done = 2;
        else
            W.sc->alpha = W.sc->rho / tot[0];
    }
}

// x += alpha p; r -= alpha q; z = r / diag; beta; convergence on ||r||
__global__ void __launch_bounds__(kBlock) k_na_x(DepIn D, NaView W) {
    if (W.sc->done) return;
    const double alpha = W.sc->alpha;
    double acc[2] = {0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.n; i += (int64_t)gridDim.x * blockDim.x) {
        D.x[i] += alpha * W.p[i];
        const double ri = W.r[i] - alpha * W.q[i];
        W.r[i] = ri;
        const double zi = ri / D.diag[i];
        W.z[i] = zi;
        acc[0] += ri * zi;
        acc[1] += ri * ri;
    }
    double tot[2];
    if (block_partials_last<2>(acc, W.partials, &W.sc->counter[0], tot) && threadIdx.x == 0) {
        W.sc->iter += 1;
        W.sc->rnorm2 = tot[1];
        W.sc->beta = tot[0] / W.sc->rho;
        W.sc->rho = tot[0];
        if (tot[1] <= W.sc->target2) W.sc->done = 1;
        else if (!isfinite(tot[1])) W.sc->done = 2;
        else if (W.sc->iter >= W.sc->maxit) W.sc->done = 3;
    }
}

// p = z + beta p
__global__ void __launch_bounds__(kBlock) k_na_p(DepIn D, NaView W) {
    if (W.sc->done) return;
    const double beta = W.sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.n; i += (int64_t)gridDim.x * blockDim.x)
        W.p[i] = W.z[i] + beta * W.p[i];
}

// (b - A x, b - A x) into sc->tmp
__global__ void __launch_bounds__(kBlock) k_na_resid(DepIn D, NaView W) {
    double acc[1] = {0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.n; i += (int64_t)gridDim.x * blockDim.x) {
        const double ri = D.rhs[i] - apply_row(D, D.x, i);
        acc[0] += ri * ri;
    }
    double tot[1];
    if (block_partials_last<1>(acc, W.partials, &W.sc->counter[0], tot) && threadIdx.x == 0) W.sc->tmp = tot[0];
}

std::mutex g_setup_mutex;
struct ScratchAddr {
    unsigned char* ptr = nullptr;
    unsigned long long ctx_id = 0;  // context the address was taken in (0: unknown)
};
ScratchAddr g_scratch_dev[64];

// The id of the current device context, 0 when there is none or the driver
// cannot say.  *known tells whether the driver offers context ids at all.
unsigned long long current_context_id(bool* known) {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess && f1 && f2) {
            get_current = reinterpret_cast<GetCurrent>(f1);
            get_id = reinterpret_cast<GetId>(f2);
        }
        resolved = true;
    }
    *known = get_current != nullptr;
    if (!get_current) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// failure messages go where pbsm3d_last_error(NULL) reads them
struct NoallocError {
    std::string msg;
    void clear() { msg.clear(); }
    NoallocError& operator=(const std::string& m) {
        msg = m;
        set_global_error(m);
        return *this;
    }
};
thread_local NoallocError g_noalloc_error;

}  // namespace
}  // namespace pbsm

using namespace pbsm;

extern "C" int pbsm3d_deposition_solve_noalloc(int64_t n_faces, const int32_t* neighbor, const double* diag,
                                               const double* off, const double* rhs, double* x, double tol,
                                               int32_t maxit, int32_t* iters, double* rel_residual) {
    g_noalloc_error.clear();
    if (n_faces <= 0 || !neighbor || !diag || !off || !rhs || !x || !(tol > 0) || maxit < 1) {
        g_noalloc_error = "invalid argument";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (n_faces > kNoAllocMaxFaces) {
        g_noalloc_error = "n_faces " + std::to_string(n_faces) + " exceeds the no-allocation limit of " +
                          std::to_string(kNoAllocMaxFaces) + " faces";
        return PBSM3D_ERR_INVALID_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        g_noalloc_error = "no current CUDA device";
        return PBSM3D_ERR_CUDA;
    }
    unsigned char* base = nullptr;
    {
        // once per device (and again after a reset of it), with that device
        // current: the device address of the scratch array (its name in host
        // code is only a stand-in)
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        bool ids = false;
        const unsigned long long ctx = current_context_id(&ids);
        ScratchAddr& a = g_scratch_dev[dev];
        if (!a.ptr || (ids && (ctx == 0 || ctx != a.ctx_id))) {
            void* ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr) {
                g_noalloc_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
                return PBSM3D_ERR_CUDA;
            }
            a.ptr = static_cast<unsigned char*>(ptr);
            a.ctx_id = current_context_id(&ids);
        }
        base = a.ptr;
    }
    NaView W = view_of(base);
    DepIn D{n_faces, neighbor, diag, off, rhs, x};
    const int grid = (int)std::min<int64_t>((n_faces + kBlock - 1) / kBlock, kNaMaxBlocks);
    cudaStream_t s = 0;
    // the reduction counters must start at zero
    if (cudaMemsetAsync(W.sc, 0, sizeof(Scalars), s) != cudaSuccess) {
        g_noalloc_error = "cudaMemsetAsync failed";
        return PBSM3D_ERR_CUDA;
    }
    auto launch_failed = [](const char* what) {
        const cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) return false;
        g_noalloc_error = std::string(what) + ": " + cudaGetErrorString(e);
        return true;
    };
    k_na_init<<<grid, kBlock, 0, s>>>(D, W, tol, maxit);
    if (launch_failed("launch of the solver's first kernel")) return PBSM3D_ERR_CUDA;
    Scalars h{};
    int it_done = 0;
    // Each batch runs 8 iterations and the device stops itself at maxit, so
    // a solve whose kernels run reports done within maxit / 8 + 1 batches;
    // a state that stops advancing is a CUDA failure, never an endless poll.
    const int64_t max_polls = (int64_t)maxit / 8 + 2;
    for (int64_t poll = 0;; ++poll) {
        if (poll >= max_polls) {
            g_noalloc_error = "deposition solver state did not advance (kernels did not run)";
            return PBSM3D_ERR_CUDA;
        }
        for (int k = 0; k < 8; ++k) {
            k_na_q<<<grid, kBlock, 0, s>>>(D, W);
            k_na_x<<<grid, kBlock, 0, s>>>(D, W);
            k_na_p<<<grid, kBlock, 0, s>>>(D, W);
        }
        if (launch_failed("launch of the solver's iteration kernels")) return PBSM3D_ERR_CUDA;
        if (cudaMemcpy(&h, W.sc, sizeof(Scalars), cudaMemcpyDeviceToHost) != cudaSuccess) {
            g_noalloc_error = std::string("CUDA error: ") + cudaGetErrorString(cudaGetLastError());
            return PBSM3D_ERR_CUDA;
        }
        if (h.done) break;
    }
    it_done = h.iter;
    const double bn2 = h.bnorm2;
    const int status = h.done;
    k_na_resid<<<grid, kBlock, 0, s>>>(D, W);
    if (launch_failed("launch of the residual kernel")) return PBSM3D_ERR_CUDA;
    if (cudaMemcpy(&h, W.sc, sizeof(Scalars), cudaMemcpyDeviceToHost) != cudaSuccess) {
        g_noalloc_error = std::string("CUDA error: ") + cudaGetErrorString(cudaGetLastError());
        return PBSM3D_ERR_CUDA;
    }
    const double rel = bn2 > 0 ? sqrt(h.tmp / bn2) : 0.0;
    if (iters) *iters = it_done;
    if (rel_residual) *rel_residual = rel;
    if (status != 1 && !(rel <= tol)) {
        g_noalloc_error = "deposition solve did not converge (relative residual " + std::to_string(rel) + ")";
        return PBSM3D_ERR_NOT_CONVERGED;
    }
    return PBSM3D_OK;
}
