// mlp.cu -- the learned warm start of the suspension solve: a per-row MLP
// 14 -> 128 -> 128 -> 128 -> 1 (ReLU) in BF16 with FP32 accumulation on the
// 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM).
//
//  * k_gemm: C[M][N] = A[M][K] * B[N][K]^T, A and B BF16 K-major, one
//    128-row tile per CTA, accumulator in TMEM, with the epilogues training
//    needs: bias + ReLU (forward), ReLU mask (backward through a layer),
//    FP32 atomic accumulation (weight gradient, split over K).
//  * k_mlp_infer: the whole network for 128-row tiles in one persistent CTA
//    per SM, weights resident in shared memory, activations never leaving
//    the SM; it writes the initial guess x0 of the Krylov solve.
//  * CUDA-core kernels for the 128 -> 1 head, the loss, bias gradients, Adam.
//
// Features of a row r = (face i, layer z) come from the assembled system and
// the previous step's solution c_prev (all normalised by the diagonal d):
//   0 (z+0.5)/L            1 log10(u_z)           2 csubl * dz * 1e3
//   3 up/|d|               4 lo/|d|               5..7 lat_j/|d|
//   8 rhs/|d| * 1e2        9 c_prev * 1e2         10 sum_j lat_j c_prev(nbr_j)/|d| * 1e2
//   11 up c_prev(above)/|d| * 1e2   12 lo c_prev(below)/|d| * 1e2
//   13 rhs(face, z=0)/|d(face, z=0)| * 1e2  (the column's saltation source)
// then standardised with the training set's mean and scale.  The network
// predicts the change of the concentration since the previous step,
// 1e2 * (c - c_prev); the guess is c_prev plus that change (where the change
// cannot be predicted the best output is ~0 and the guess falls back to the
// previous step's field).
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <random>
#include <vector>

#include "pbsm3d_internal.cuh"
#include "tc_sm103.cuh"

namespace pbsm {

constexpr int kFeat = 14;
constexpr int kHid = 128;
constexpr float kCScale = 100.0f;
constexpr unsigned long long kMmaWaitNs = 1000000000ull;  // 1 s

namespace {

using bf16 = __nv_bfloat16;

enum { EPI_F32 = 0, EPI_FWD = 1, EPI_BWDD = 2, EPI_WGRAD = 3 };

struct GemmArgs {
    const bf16* A;
    int lda;
    const bf16* B;
    int ldb;
    int M, K;
    int k_chunk;  // K per CTA (blockIdx.y selects the chunk); multiple of 64, or 16 when K == 16
    const float* bias;
    const bf16* mask;
    int ldm;
    bf16* out;
    int ldo;
    bf16* outT;
    int ldoT;
    float* outF;  // EPI_F32: [M][N]; EPI_WGRAD: atomically accumulated [M][N]
    int* err;
};

// Load rows [r0, r0+R) x 16-byte chunks [0, nch) of a K-major BF16 matrix
// (chunk c = columns k0 + 8c .. +7) into a SW128 tile.
__device__ __forceinline__ void load_tile(unsigned char* tile, const bf16* src, int ld, int r0, int R, int k0,
                                          int nch) {
    const int total = R * nch;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int r = idx / nch, c = idx % nch;
        const uint4 v = *reinterpret_cast<const uint4*>(src + (size_t)(r0 + r) * ld + k0 + c * 8);
        *reinterpret_cast<uint4*>(tile + tc::sw128_chunk(r, c, R)) = v;
    }
}

template <int N, int EPI>
__global__ void __launch_bounds__(128) k_gemm(GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* tA = base;                // 128 x 64 bf16 = 16 KB
    unsigned char* tB = base + 16384;        // N x 64 bf16
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t tmem_slot;
    constexpr int kCols = N < 32 ? 32 : N;
    const int warp = threadIdx.x >> 5;
    const int m0 = blockIdx.x * 128;
    const int kbeg = blockIdx.y * g.k_chunk;
    const int kend = min(g.K, kbeg + g.k_chunk);
    const uint32_t mb = tc::smem_u32(&mbar);
    if (threadIdx.x == 0) tc::mbar_init(mb, 1);
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_u32(&tmem_slot), kCols);
        tc::tmem_relinquish();
    }
    __syncthreads();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(128, N);
    uint32_t phase = 0;
    bool ok = true;
    bool first = true;
    for (int k0 = kbeg; k0 < kend && ok; k0 += 64) {
        const int kc = min(64, kend - k0);  // 64, or 16 for the K = 16 layer
        const int nch = kc / 8;
        load_tile(tA, g.A, g.lda, m0, 128, k0, nch);
        load_tile(tB, g.B, g.ldb, 0, N, k0, nch);
        tc::fence_proxy_async();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc::fence_after_sync();
            const uint32_t sa = tc::smem_u32(tA), sb = tc::smem_u32(tB);
            for (int s = 0; s < kc / 16; ++s) {
                tc::mma_bf16(tmem, tc::desc_kstep(sa, s, 128), tc::desc_kstep(sb, s, N), idesc, first ? 0u : 1u);
                first = false;
            }
            tc::mma_commit(mb);
        }
        __syncwarp();
        const bool waited = tc::mbar_wait(mb, phase, kMmaWaitNs);
        ok = __syncthreads_and(waited) != 0;  // uniform across the CTA
        if (!ok) {
            if (threadIdx.x == 0) atomicExch(g.err, 1);
            tc::mbar_wait(mb, phase, kMmaWaitNs);  // give in-flight MMAs a second bounded chance
        }
        phase ^= 1u;
    }
    tc::fence_after_sync();
    if (ok) {
        const int m = m0 + threadIdx.x;  // this thread's TMEM lane = row
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += 32) {
            float v[32];
            tc::tmem_ld32(lane_addr + (uint32_t)c0, v);
            const int nv = min(32, N - c0);
            if (EPI == EPI_F32) {
                for (int j = 0; j < nv; ++j) g.outF[(size_t)m * N + c0 + j] = v[j];
            } else if (EPI == EPI_WGRAD) {
                for (int j = 0; j < nv; ++j) atomicAdd(&g.outF[(size_t)m * N + c0 + j], v[j]);
            } else {
                for (int j = 0; j < nv; ++j) {
                    const int n = c0 + j;
                    float y;
                    if (EPI == EPI_FWD) {
                        y = fmaxf(v[j] + g.bias[n], 0.0f);
                    } else {
                        const float hm = __bfloat162float(g.mask[(size_t)m * g.ldm + n]);
                        y = hm > 0.0f ? v[j] : 0.0f;
                    }
                    const bf16 yb = __float2bfloat16_rn(y);
                    g.out[(size_t)m * g.ldo + n] = yb;
                    if (g.outT) g.outT[(size_t)n * g.ldoT + m] = yb;
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// ---------------------------------------------------------------- features
struct FeatSrc {
    const double* band;   // [6][R]
    const double* rhs;    // [R]
    const double* u_z;    // [R]
    const double* csubl;  // [R]
    const double* cprev;  // [R]
    const int32_t* nbr;   // [3][Tp]
    int64_t Tp, R;
    int L;
    double dz;
};

// The features are BF16 inputs after standardisation, so they are formed in
// FP32 from the FP64 system (one conversion per value; FP64 divisions and
// log10 would cost the GB300's slow FP64 pipe ~80 instructions a row).  They
// come in two halves, features 0-7 and 8-13, so that the fused inference can
// give a row's halves to two threads; the training path forms both.
__device__ __forceinline__ float feat_inv_diag(const FeatSrc& s, int64_t r) {
    const float d = (float)s.band[r];
    const float ad = fabsf(d) > 0.0f ? fabsf(d) : 1.0f;
    return 1.0f / ad;
}

__device__ __forceinline__ void row_features_lo(const FeatSrc& s, int64_t i, int z, float* f) {
    const int64_t r = (int64_t)z * s.Tp + i;
    const float inv = feat_inv_diag(s, r);
    f[0] = (z + 0.5f) / (float)s.L;
    f[1] = log10f(fmaxf((float)s.u_z[r], 1e-3f));
    f[2] = (float)s.csubl[r] * ((float)s.dz * 1e3f);
    f[3] = (float)s.band[5 * s.R + r] * inv;
    f[4] = (float)s.band[4 * s.R + r] * inv;
    for (int j = 0; j < 3; ++j) f[5 + j] = (float)s.band[(1 + j) * s.R + r] * inv;
}

__device__ __forceinline__ void row_features_hi(const FeatSrc& s, int64_t i, int z, float* f) {
    const int64_t r = (int64_t)z * s.Tp + i;
    const float inv = feat_inv_diag(s, r);
    const float up = (float)s.band[5 * s.R + r], lo = (float)s.band[4 * s.R + r];
    float latc = 0.0f;
    for (int j = 0; j < 3; ++j) {
        const int32_t nb = s.nbr[j * s.Tp + i];
        if (nb >= 0) latc += (float)s.band[(1 + j) * s.R + r] * (float)s.cprev[(int64_t)z * s.Tp + nb];
    }
    const float above = z + 1 < s.L ? (float)s.cprev[r + s.Tp] : 0.0f;
    const float below = z > 0 ? (float)s.cprev[r - s.Tp] : 0.0f;
    const float b0 = fabsf((float)s.band[i]);
    const float d0 = b0 > 0.0f ? b0 : 1.0f;
    f[0] = (float)s.rhs[r] * inv * kCScale;
    f[1] = (float)s.cprev[r] * kCScale;
    f[2] = latc * inv * kCScale;
    f[3] = up * above * inv * kCScale;
    f[4] = lo * below * inv * kCScale;
    f[5] = (float)s.rhs[i] / d0 * kCScale;
}

__device__ __forceinline__ void row_features(const FeatSrc& s, int64_t i, int z, float (&f)[kFeat]) {
    row_features_lo(s, i, z, f);
    row_features_hi(s, i, z, f + 8);
}

// features [rows][14] (raw, un-standardised) and target [rows] = c * 1e2, rows in reference order
__global__ void k_features(FeatSrc s, const double* x_now, int64_t T, float* feat, float* target) {
    const int64_t n = T * s.L;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int z = (int)(q / T);
        const int64_t i = q - (int64_t)z * T;
        float f[kFeat];
        row_features(s, i, z, f);
        for (int k = 0; k < kFeat; ++k) feat[q * kFeat + k] = f[k];
        // the network learns the step-to-step change of the concentration
        const int64_t r = (int64_t)z * s.Tp + i;
        if (target) target[q] = (float)((x_now[r] - s.cprev[r]) * kCScale);
    }
}

// ---------------------------------------------------------------- fused inference
struct InferArgs {
    FeatSrc src;
    int64_t T;
    const bf16* W0;  // [128][16]
    const bf16* W1;  // [128][128]
    const bf16* W2;
    const float* b0;
    const float* b1;
    const float* b2;
    const float* w3;
    float b3;
    const float* fmean;
    const float* fscale;
    double* x0;  // [R] device layout
    int* err;
};

constexpr int kGroups = 2, kGroupThreads = 256, kInferThreads = kGroups * kGroupThreads;
// the weights, then each group's X (128 x 16, 128-byte rows) and H (128 x 128)
constexpr int kInferSmem = 16384 + 32768 + 32768 + kGroups * (16384 + 32768) + 1024;

// Weights -> SW128 tiles (R = 128 rows).  W0 has K = 16 (2 chunks per row).
__device__ __forceinline__ void stage_weights(unsigned char* t, const bf16* W, int K) {
    load_tile(t, W, K, 0, 128, 0, K / 8);
}

// Two groups of 256 threads, each with its own 128-row tile in flight: its
// own X and H buffers in shared memory, its own 128 TMEM columns, mbarrier and
// named barrier, the weights shared.  While one group forms features or runs
// its epilogue on the CUDA cores, the other's MMAs can run.  Within a group,
// warps w and w + 4 read the same TMEM lanes (rows 32 (w % 4) ...): each of a
// row's two threads forms half its features and takes half the epilogue's 128
// columns.  (One 128-thread tile at a time stalled on fixed-latency waits with
// the tensor pipe ~6% busy.)
__device__ __forceinline__ void group_sync(int grp) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(kGroupThreads) : "memory");
}

__global__ void __launch_bounds__(kInferThreads) k_mlp_infer(InferArgs a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sW0 = base;
    unsigned char* sW1 = sW0 + 16384;
    unsigned char* sW2 = sW1 + 32768;
    __shared__ __align__(8) unsigned long long mbar[kGroups];
    __shared__ uint32_t tmem_slot;
    __shared__ float sb[3][kHid];
    __shared__ float sw3[kHid];
    __shared__ float yh[kGroups][128];  // the second column half's head partial per row
    __shared__ int s_ok[kGroups];
    const int warp = threadIdx.x >> 5;
    const int grp = threadIdx.x / kGroupThreads, gt = threadIdx.x % kGroupThreads, gwarp = gt >> 5;
    const int row = gt & 127, half = gwarp >> 2;  // this thread's tile row; column half
    unsigned char* sX = sW2 + 32768 + grp * (16384 + 32768);
    unsigned char* sH = sX + 16384;
    const uint32_t mb = tc::smem_u32(&mbar[grp]);
    if (threadIdx.x == 0)
        for (int g = 0; g < kGroups; ++g) tc::mbar_init(tc::smem_u32(&mbar[g]), 1);
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_u32(&tmem_slot), 128 * kGroups);
        tc::tmem_relinquish();
    }
    stage_weights(sW0, a.W0, 16);
    stage_weights(sW1, a.W1, kHid);
    stage_weights(sW2, a.W2, kHid);
    for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
        sb[0][k] = a.b0[k];
        sb[1][k] = a.b1[k];
        sb[2][k] = a.b2[k];
        sw3[k] = a.w3[k];
    }
    __syncthreads();
    const uint32_t tmem = tmem_slot + (uint32_t)(grp * 128);  // this group's columns
    const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t idesc = tc::idesc_bf16(128, kHid);
    const uint32_t aX = tc::smem_u32(sX), aH = tc::smem_u32(sH);
    const uint32_t aW0 = tc::smem_u32(sW0), aW1 = tc::smem_u32(sW1), aW2 = tc::smem_u32(sW2);
    const int64_t rows = a.T * a.src.L;
    const int64_t ntiles = (rows + 127) / 128;
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t tile = (int64_t)blockIdx.x * kGroups + grp; tile < ntiles && ok;
         tile += (int64_t)gridDim.x * kGroups) {
        const int64_t q = tile * 128 + row;  // reference-order row of this thread
        const bool valid = q < rows;
        int z = 0;
        int64_t i = 0;
        if (valid) {
            z = (int)(q / a.T);
            i = q - (int64_t)z * a.T;
        }
        // features -> standardised -> bf16 -> X row: this thread's half of
        // the 16 columns (features 0-7, or 8-13 and two zero pads), one chunk
        {
            float f[8];
            if (valid) {
                if (half == 0)
                    row_features_lo(a.src, i, z, f);
                else
                    row_features_hi(a.src, i, z, f);
            }
            __align__(16) bf16 xb[8];
            for (int k = 0; k < 8; ++k) {
                const int col = half * 8 + k;
                float v = 0.0f;
                if (valid && col < kFeat) v = (f[k] - a.fmean[col]) * a.fscale[col];
                xb[k] = __float2bfloat16_rn(v);
            }
            *reinterpret_cast<uint4*>(sX + tc::sw128_chunk(row, half, 128)) = *reinterpret_cast<const uint4*>(xb);
        }
        float y = 0.0f;
        for (int layer = 0; layer < 3 && ok; ++layer) {
            tc::fence_proxy_async();
            tc::fence_before_sync();
            group_sync(grp);
            if (gt == 0) {
                tc::fence_after_sync();
                if (layer == 0) {
                    tc::mma_bf16(tmem, tc::desc_kstep(aX, 0, 128), tc::desc_kstep(aW0, 0, 128), idesc, 0u);
                } else {
                    const uint32_t aw = layer == 1 ? aW1 : aW2;
                    for (int s = 0; s < kHid / 16; ++s)
                        tc::mma_bf16(tmem, tc::desc_kstep(aH, s, 128), tc::desc_kstep(aw, s, 128), idesc,
                                     s > 0 ? 1u : 0u);
                }
                tc::mma_commit(mb);
            }
            __syncwarp();
            const bool waited = tc::mbar_wait(mb, phase, kMmaWaitNs);
            // uniform across the group: every thread leaves together on a timeout
            if (gt == 0) s_ok[grp] = 1;
            group_sync(grp);
            if (!waited) s_ok[grp] = 0;
            group_sync(grp);
            ok = s_ok[grp] != 0;
            group_sync(grp);
            if (!ok) {
                if (gt == 0) atomicExch(a.err, 1);
                tc::mbar_wait(mb, phase, kMmaWaitNs);
                break;
            }
            phase ^= 1u;
            tc::fence_after_sync();
            // epilogue, this thread's column half: bias + ReLU; layers 0, 1 -> H
            // (bf16); layer 2 -> head dot
#pragma unroll 1
            for (int c0 = half * (kHid / 2); c0 < (half + 1) * (kHid / 2); c0 += 32) {
                float v[32];
                tc::tmem_ld32(lane_addr + (uint32_t)c0, v);
                if (layer < 2) {
                    __align__(16) bf16 hb[32];
#pragma unroll
                    for (int j = 0; j < 32; ++j) hb[j] = __float2bfloat16_rn(fmaxf(v[j] + sb[layer][c0 + j], 0.0f));
                    const uint4* hs = reinterpret_cast<const uint4*>(hb);
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc)
                        *reinterpret_cast<uint4*>(sH + tc::sw128_chunk(row, c0 / 8 + cc, 128)) = hs[cc];
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j) y += fmaxf(v[j] + sb[2][c0 + j], 0.0f) * sw3[c0 + j];
                }
            }
        }
        // head: the first half's partial plus the second's, in that order
        if (half == 1) yh[grp][row] = y;
        group_sync(grp);
        if (ok && valid && half == 0) {
            const int64_t r = (int64_t)z * a.src.Tp + i;
            a.x0[r] = a.src.cprev[r] + (double)((y + yh[grp][row] + a.b3) / kCScale);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem_slot, 128 * kGroups);
}

// ---------------------------------------------------------------- training kernels
// batch: rows idx[0..B) of feat/target -> standardised X [B][16] and X^T [16][B] (bf16), t [B]
__global__ void k_pack_batch(const float* feat, const float* target, const int64_t* idx, int B,
                             const float* fmean, const float* fscale, bf16* X, bf16* XT, float* t) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        const int64_t q = idx[b];
        for (int k = 0; k < 16; ++k) {
            const float v = k < kFeat ? (feat[q * kFeat + k] - fmean[k]) * fscale[k] : 0.0f;
            const bf16 vb = __float2bfloat16_rn(v);
            X[(size_t)b * 16 + k] = vb;
            XT[(size_t)k * B + b] = vb;
        }
        t[b] = target[q];
    }
}

// head: y = H3 w3 + b3, loss 0.5 mean (y-t)^2, dY = (y-t)/B, dH3 = dY w3 * (H3 > 0),
// dw3 += dY H3, db3 += dY, loss_acc += 0.5 (y-t)^2 / B
__global__ void k_head(const bf16* H3, const float* w3, float b3, const float* t, int B, bf16* dH3, bf16* dH3T,
                       float* dw3, float* db3, float* loss_acc, float* y_out) {
    __shared__ float sw[kHid];
    __shared__ float sdw[kHid];
    for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
        sw[k] = w3[k];
        sdw[k] = 0.0f;
    }
    __syncthreads();
    float lsum = 0.0f, dbsum = 0.0f;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        float y = b3;
        for (int k = 0; k < kHid; ++k) y += __bfloat162float(H3[(size_t)b * kHid + k]) * sw[k];
        if (y_out) y_out[b] = y;
        const float e = y - t[b];
        lsum += 0.5f * e * e / B;
        const float dy = e / B;
        dbsum += dy;
        for (int k = 0; k < kHid; ++k) {
            const float h = __bfloat162float(H3[(size_t)b * kHid + k]);
            const bf16 g = __float2bfloat16_rn(h > 0.0f ? dy * sw[k] : 0.0f);
            dH3[(size_t)b * kHid + k] = g;
            dH3T[(size_t)k * B + b] = g;
            atomicAdd(&sdw[k], dy * h);
        }
    }
    atomicAdd(loss_acc, lsum);
    atomicAdd(db3, dbsum);
    __syncthreads();
    for (int k = threadIdx.x; k < kHid; k += blockDim.x) atomicAdd(&dw3[k], sdw[k]);
}

// db[n] += sum_b dHT[n][b]
__global__ void k_bias_grad(const bf16* dHT, int B, float* db) {
    const int n = blockIdx.x;
    float s = 0.0f;
    for (int b = threadIdx.x; b < B; b += blockDim.x) s += __bfloat162float(dHT[(size_t)n * B + b]);
    s = warp_sum(s);
    __shared__ float sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        db[n] += t;
    }
}

// Adam on FP32 master parameters; g is zeroed for the next batch
__global__ void k_adam(float* p, float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const float gk = g[k];
        const float mk = b1 * m[k] + (1 - b1) * gk;
        const float vk = b2 * v[k] + (1 - b2) * gk * gk;
        m[k] = mk;
        v[k] = vk;
        p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
        g[k] = 0.0f;
    }
}

// bf16 copies: W [out][in] and W^T [in][out] (in padded to ld_in)
__global__ void k_to_bf16(const float* W, int out, int in, int ld_in, bf16* Wb, bf16* WbT) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < out * ld_in; k += gridDim.x * blockDim.x) {
        const int o = k / ld_in, c = k % ld_in;
        const bf16 v = __float2bfloat16_rn(c < in ? W[o * in + c] : 0.0f);
        Wb[(size_t)o * ld_in + c] = v;
        if (WbT) WbT[(size_t)c * out + o] = v;
    }
}

// dW0 (padded [128][16]) -> the packed gradient [128][14]
__global__ void k_fold_w0(const float* dW0pad, float* gW0) {
    const int o = blockIdx.x;
    for (int k = threadIdx.x; k < kFeat; k += blockDim.x) gW0[o * kFeat + k] += dW0pad[o * 16 + k];
}

}  // namespace

// ---------------------------------------------------------------- host side
template <int N, int EPI>
static cudaError_t launch_gemm(const GemmArgs& g, int splits, cudaStream_t s) {
    const int smem = 16384 + N * 128 + 1024;
    cudaError_t e = cudaFuncSetAttribute(k_gemm<N, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_gemm<N, EPI><<<dim3(g.M / 128, splits), 128, smem, s>>>(g);
    return cudaGetLastError();
}

struct MlpTrainer {
    int B;  // batch rows (multiple of 128)
    cudaStream_t s;
    // fp32 master parameters, gradients and Adam moments in one block each:
    // W0[128*14] b0[128] W1[128*128] b1 W2 b2 w3[128] b3[1]
    float *P, *G, *Mo, *Vo;
    int np;
    bf16 *W0b, *W1b, *W1bT, *W2b, *W2bT;  // bf16 weights (W0 padded to 16 inputs)
    bf16 *X, *XT, *H1, *H1T, *H2, *H2T, *H3, *H3T, *dH3, *dH3T, *dH2, *dH2T, *dH1, *dH1T;
    float *t, *loss, *y;
    float* dW0pad;  // [128][16] gradient of the padded first layer
    float *fmean, *fscale;
    int64_t* idx;
    int* err;
    std::vector<void*> allocs;
    int step = 0;
};

static const int kOffW0 = 0, kOffB0 = kOffW0 + kHid * kFeat, kOffW1 = kOffB0 + kHid, kOffB1 = kOffW1 + kHid * kHid,
                 kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid,
                 kOffB3 = kOffW3 + kHid, kNumParams = kOffB3 + 1;

template <typename T>
static T* talloc(MlpTrainer& t, size_t n, bool& ok) {
    void* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        ok = false;
        return nullptr;
    }
    t.allocs.push_back(p);
    return static_cast<T*>(p);
}

static void trainer_free(MlpTrainer* t) {
    if (!t) return;
    for (void* p : t->allocs) cudaFree(p);
    if (t->s) cudaStreamDestroy(t->s);
    delete t;
}

static MlpTrainer* trainer_new(int B) {
    auto* t = new MlpTrainer();
    t->B = B;
    t->np = kNumParams;
    bool ok = cudaStreamCreateWithFlags(&t->s, cudaStreamNonBlocking) == cudaSuccess;
    t->P = talloc<float>(*t, kNumParams, ok);
    t->G = talloc<float>(*t, kNumParams, ok);
    t->Mo = talloc<float>(*t, kNumParams, ok);
    t->Vo = talloc<float>(*t, kNumParams, ok);
    t->W0b = talloc<bf16>(*t, kHid * 16, ok);
    t->W1b = talloc<bf16>(*t, kHid * kHid, ok);
    t->W1bT = talloc<bf16>(*t, kHid * kHid, ok);
    t->W2b = talloc<bf16>(*t, kHid * kHid, ok);
    t->W2bT = talloc<bf16>(*t, kHid * kHid, ok);
    const size_t act = (size_t)B * kHid;
    t->X = talloc<bf16>(*t, (size_t)B * 16, ok);
    t->XT = talloc<bf16>(*t, (size_t)B * 16, ok);
    bf16** bufs[] = {&t->H1, &t->H1T, &t->H2, &t->H2T, &t->H3, &t->H3T, &t->dH3, &t->dH3T, &t->dH2, &t->dH2T,
                     &t->dH1, &t->dH1T};
    for (bf16** b : bufs) *b = talloc<bf16>(*t, act, ok);
    t->t = talloc<float>(*t, B, ok);
    t->y = talloc<float>(*t, B, ok);
    t->loss = talloc<float>(*t, 1, ok);
    t->dW0pad = talloc<float>(*t, kHid * 16, ok);
    t->fmean = talloc<float>(*t, kFeat, ok);
    t->fscale = talloc<float>(*t, kFeat, ok);
    t->idx = talloc<int64_t>(*t, B, ok);
    t->err = talloc<int>(*t, 1, ok);
    if (!ok) {
        trainer_free(t);
        return nullptr;
    }
    cudaMemsetAsync(t->G, 0, kNumParams * 4, t->s);
    cudaMemsetAsync(t->Mo, 0, kNumParams * 4, t->s);
    cudaMemsetAsync(t->Vo, 0, kNumParams * 4, t->s);
    cudaMemsetAsync(t->err, 0, 4, t->s);
    return t;
}

static void refresh_bf16(MlpTrainer* t) {
    k_to_bf16<<<64, 256, 0, t->s>>>(t->P + kOffW0, kHid, kFeat, 16, t->W0b, nullptr);
    k_to_bf16<<<64, 256, 0, t->s>>>(t->P + kOffW1, kHid, kHid, kHid, t->W1b, t->W1bT);
    k_to_bf16<<<64, 256, 0, t->s>>>(t->P + kOffW2, kHid, kHid, kHid, t->W2b, t->W2bT);
}

// forward + backward of one packed batch (X, XT, t already on device); gradients accumulate into G
static cudaError_t fwd_bwd(MlpTrainer* t, float b3) {
    const int B = t->B;
    cudaStream_t s = t->s;
    cudaError_t e;
    GemmArgs g{};
    g.err = t->err;
    // forward
    g = GemmArgs{t->X, 16, t->W0b, 16, B, 16, 16, t->P + kOffB0, nullptr, 0, t->H1, kHid, t->H1T, B, nullptr, t->err};
    if ((e = launch_gemm<kHid, EPI_FWD>(g, 1, s)) != cudaSuccess) return e;
    g = GemmArgs{t->H1, kHid, t->W1b, kHid, B, kHid, kHid, t->P + kOffB1, nullptr, 0, t->H2, kHid, t->H2T, B, nullptr,
                 t->err};
    if ((e = launch_gemm<kHid, EPI_FWD>(g, 1, s)) != cudaSuccess) return e;
    g = GemmArgs{t->H2, kHid, t->W2b, kHid, B, kHid, kHid, t->P + kOffB2, nullptr, 0, t->H3, kHid, t->H3T, B, nullptr,
                 t->err};
    if ((e = launch_gemm<kHid, EPI_FWD>(g, 1, s)) != cudaSuccess) return e;
    // head
    k_head<<<std::min(148, (B + 255) / 256), 256, 0, s>>>(t->H3, t->P + kOffW3, b3, t->t, B, t->dH3, t->dH3T,
                                                          t->G + kOffW3, t->G + kOffB3, t->loss, t->y);
    // layer 2: dW2 = dH3^T H2 (split over batch rows), dH2 = (dH3 W2) * (H2 > 0)
    const int kc = std::min(B, 1024);
    const int splits = B / kc;
    g = GemmArgs{t->dH3T, B, t->H2T, B, kHid, B, kc, nullptr, nullptr, 0, nullptr, 0, nullptr, 0, t->G + kOffW2,
                 t->err};
    if ((e = launch_gemm<kHid, EPI_WGRAD>(g, splits, s)) != cudaSuccess) return e;
    k_bias_grad<<<kHid, 256, 0, s>>>(t->dH3T, B, t->G + kOffB2);
    g = GemmArgs{t->dH3, kHid, t->W2bT, kHid, B, kHid, kHid, nullptr, t->H2, kHid, t->dH2, kHid, t->dH2T, B, nullptr,
                 t->err};
    if ((e = launch_gemm<kHid, EPI_BWDD>(g, 1, s)) != cudaSuccess) return e;
    // layer 1
    g = GemmArgs{t->dH2T, B, t->H1T, B, kHid, B, kc, nullptr, nullptr, 0, nullptr, 0, nullptr, 0, t->G + kOffW1,
                 t->err};
    if ((e = launch_gemm<kHid, EPI_WGRAD>(g, splits, s)) != cudaSuccess) return e;
    k_bias_grad<<<kHid, 256, 0, s>>>(t->dH2T, B, t->G + kOffB1);
    g = GemmArgs{t->dH2, kHid, t->W1bT, kHid, B, kHid, kHid, nullptr, t->H1, kHid, t->dH1, kHid, t->dH1T, B, nullptr,
                 t->err};
    if ((e = launch_gemm<kHid, EPI_BWDD>(g, 1, s)) != cudaSuccess) return e;
    // layer 0: dW0 = dH1^T X  (N = 16 inputs incl. 2 zero pads), into a padded buffer
    g = GemmArgs{t->dH1T, B, t->XT, B, kHid, B, kc, nullptr, nullptr, 0, nullptr, 0, nullptr, 0, t->dW0pad,
                 t->err};
    if ((e = launch_gemm<16, EPI_WGRAD>(g, splits, s)) != cudaSuccess) return e;
    k_bias_grad<<<kHid, 256, 0, s>>>(t->dH1T, B, t->G + kOffB0);
    k_fold_w0<<<kHid, 32, 0, s>>>(t->dW0pad, t->G + kOffW0);
    return cudaGetLastError();
}

// ---- inference and features in a context
static FeatSrc feat_src(Ctx& c) {
    return FeatSrc{c.A.band, c.A.rhs, c.A.u_z, c.A.csubl, c.x_prev, c.F.nbr, c.P.Tp, c.P.R, c.P.L, c.P.dz};
}

int launch_mlp_infer(Ctx& c, cudaStream_t s, double* x0) {
    if (!c.mlp_loaded) {
        c.err = "learned warm start requested but no MLP loaded (pbsm3d_set_mlp)";
        return PBSM3D_ERR_INVALID_ARG;
    }
    const bf16* w = static_cast<const bf16*>(c.mlp_w);
    const float* f = c.mlp_f;
    InferArgs a{feat_src(c), c.P.T, w, w + kHid * 16, w + kHid * 16 + kHid * kHid, f, f + kHid, f + 2 * kHid,
                f + 3 * kHid, c.mlp_b3, f + 4 * kHid + 1, f + 4 * kHid + 1 + kFeat, x0, (int*)&c.gbar->err};
    PBSM_CUDA_TRY(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t tiles = (c.P.T * c.P.L + 127) / 128;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((tiles + kGroups - 1) / kGroups, sms));
    PBSM_CUDA_TRY(cudaMemsetAsync(&c.gbar->err, 0, sizeof(int), s));
    prof_begin(c, s);
    k_mlp_infer<<<grid, kInferThreads, kInferSmem, s>>>(a);
    // per row: 14 feature inputs (~12 doubles read) + x0 written; weights once per CTA
    prof_end(c, s, PBSM3D_K_MLP, c.P.T * c.P.L * (12 * 8 + 8));
    PBSM_CUDA_TRY(cudaGetLastError());
    return 0;
}

int mlp_features(Ctx& c, float* feat_dev, float* target_dev) {
    k_features<<<c.grid_faces, kBlock, 0, c.stream>>>(feat_src(c), c.A.x, c.P.T, feat_dev, target_dev);
    PBSM_CUDA_TRY(cudaGetLastError());
    return 0;
}

int mlp_load(Ctx& c, const float* params, const float* fmean, const float* fscale) {
    if (!c.mlp_w) {
        PBSM_CUDA_TRY(cudaMalloc(&c.mlp_w, (size_t)(kHid * 16 + 2 * kHid * kHid) * 2));
        c.allocations.push_back(c.mlp_w);
        void* f = nullptr;
        PBSM_CUDA_TRY(cudaMalloc(&f, (size_t)(4 * kHid + 1 + 2 * kFeat) * 4));
        c.allocations.push_back(f);
        c.mlp_f = static_cast<float*>(f);
    }
    std::vector<bf16> w(kHid * 16 + 2 * kHid * kHid);
    for (int o = 0; o < kHid; ++o)
        for (int k = 0; k < 16; ++k) w[o * 16 + k] = __float2bfloat16_rn(k < kFeat ? params[kOffW0 + o * kFeat + k] : 0.f);
    for (int q = 0; q < kHid * kHid; ++q) {
        w[kHid * 16 + q] = __float2bfloat16_rn(params[kOffW1 + q]);
        w[kHid * 16 + kHid * kHid + q] = __float2bfloat16_rn(params[kOffW2 + q]);
    }
    std::vector<float> f(4 * kHid + 1 + 2 * kFeat);
    for (int k = 0; k < kHid; ++k) {
        f[k] = params[kOffB0 + k];
        f[kHid + k] = params[kOffB1 + k];
        f[2 * kHid + k] = params[kOffB2 + k];
        f[3 * kHid + k] = params[kOffW3 + k];
    }
    f[4 * kHid] = params[kOffB3];
    for (int k = 0; k < kFeat; ++k) {
        f[4 * kHid + 1 + k] = fmean[k];
        f[4 * kHid + 1 + kFeat + k] = fscale[k];
    }
    PBSM_CUDA_TRY(cudaMemcpy(c.mlp_w, w.data(), w.size() * 2, cudaMemcpyHostToDevice));
    PBSM_CUDA_TRY(cudaMemcpy(c.mlp_f, f.data(), f.size() * 4, cudaMemcpyHostToDevice));
    c.mlp_b3 = params[kOffB3];
    c.mlp_loaded = true;
    return 0;
}

}  // namespace pbsm

using namespace pbsm;

struct pbsm3d_mlp_trainer {
    MlpTrainer* t;
};

extern "C" {

int pbsm3d_mlp_num_params(void) { return kNumParams; }

int pbsm3d_mlp_trainer_create(int32_t batch, const float* params, const float* feat_mean, const float* feat_scale,
                              pbsm3d_mlp_trainer** out) {
    if (!out || !params || !feat_mean || !feat_scale || batch < 128 || batch % 128 != 0 ||
        (batch > 1024 && batch % 1024 != 0)) {
        set_global_error("trainer: batch must be a multiple of 128 (and of 1024 above 1024)");
        return PBSM3D_ERR_INVALID_ARG;
    }
    MlpTrainer* t = trainer_new(batch);
    if (!t) {
        set_global_error("trainer: out of device memory");
        return PBSM3D_ERR_OUT_OF_MEMORY;
    }
    cudaMemcpyAsync(t->P, params, kNumParams * 4, cudaMemcpyHostToDevice, t->s);
    cudaMemcpyAsync(t->fmean, feat_mean, kFeat * 4, cudaMemcpyHostToDevice, t->s);
    cudaMemcpyAsync(t->fscale, feat_scale, kFeat * 4, cudaMemcpyHostToDevice, t->s);
    refresh_bf16(t);
    if (cudaStreamSynchronize(t->s) != cudaSuccess) {
        set_global_error("trainer: CUDA error at create");
        trainer_free(t);
        return PBSM3D_ERR_CUDA;
    }
    *out = new pbsm3d_mlp_trainer{t};
    return PBSM3D_OK;
}

void pbsm3d_mlp_trainer_destroy(pbsm3d_mlp_trainer* h) {
    if (!h) return;
    cudaStreamSynchronize(h->t->s);
    trainer_free(h->t);
    delete h;
}

int pbsm3d_mlp_get_params(pbsm3d_mlp_trainer* h, float* params) {
    if (!h || !params) return PBSM3D_ERR_INVALID_ARG;
    if (cudaMemcpyAsync(params, h->t->P, kNumParams * 4, cudaMemcpyDeviceToHost, h->t->s) != cudaSuccess ||
        cudaStreamSynchronize(h->t->s) != cudaSuccess)
        return PBSM3D_ERR_CUDA;
    return PBSM3D_OK;
}

// One forward/backward pass over host rows (exactly `batch` of them):
// gradients of 0.5 mean((y - t)^2) w.r.t. every parameter, loss and outputs.
int pbsm3d_mlp_grad(pbsm3d_mlp_trainer* h, const float* feat, const float* target, float* grads, float* loss,
                    float* y) {
    if (!h || !feat || !target || !grads) return PBSM3D_ERR_INVALID_ARG;
    MlpTrainer* t = h->t;
    const int B = t->B;
    cudaStream_t s = t->s;
    float* dfeat = nullptr;
    float* dtarget = nullptr;
    if (cudaMalloc(&dfeat, (size_t)B * kFeat * 4) != cudaSuccess) return PBSM3D_ERR_OUT_OF_MEMORY;
    if (cudaMalloc(&dtarget, (size_t)B * 4) != cudaSuccess) {
        cudaFree(dfeat);
        return PBSM3D_ERR_OUT_OF_MEMORY;
    }
    std::vector<int64_t> idx(B);
    for (int b = 0; b < B; ++b) idx[b] = b;
    float b3 = 0;
    cudaMemcpy(&b3, t->P + kOffB3, 4, cudaMemcpyDeviceToHost);
    cudaMemcpyAsync(dfeat, feat, (size_t)B * kFeat * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dtarget, target, (size_t)B * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(t->idx, idx.data(), (size_t)B * 8, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(t->G, 0, kNumParams * 4, s);
    cudaMemsetAsync(t->dW0pad, 0, kHid * 16 * 4, s);
    cudaMemsetAsync(t->loss, 0, 4, s);
    k_pack_batch<<<(B + 255) / 256, 256, 0, s>>>(dfeat, dtarget, t->idx, B, t->fmean, t->fscale, t->X, t->XT, t->t);
    cudaError_t e = fwd_bwd(t, b3);
    int err = 0;
    if (e == cudaSuccess) {
        cudaMemcpyAsync(grads, t->G, kNumParams * 4, cudaMemcpyDeviceToHost, s);
        if (loss) cudaMemcpyAsync(loss, t->loss, 4, cudaMemcpyDeviceToHost, s);
        if (y) cudaMemcpyAsync(y, t->y, (size_t)B * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&err, t->err, 4, cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
    }
    cudaMemsetAsync(t->G, 0, kNumParams * 4, s);
    cudaStreamSynchronize(s);
    cudaFree(dfeat);
    cudaFree(dtarget);
    if (e != cudaSuccess || err) {
        set_global_error(err ? "mlp: tensor-core wait timed out" : cudaGetErrorString(e));
        return PBSM3D_ERR_CUDA;
    }
    return PBSM3D_OK;
}

// Adam training on device rows: `steps` minibatches drawn uniformly (seeded)
// from feat [rows][14] / target [rows] (device pointers).
int pbsm3d_mlp_train(pbsm3d_mlp_trainer* h, const float* feat, const float* target, int64_t rows, int32_t steps,
                     float lr, uint64_t seed, float* loss_per_step) {
    if (!h || !feat || !target || rows < 1 || steps < 1 || !(lr > 0)) return PBSM3D_ERR_INVALID_ARG;
    MlpTrainer* t = h->t;
    const int B = t->B;
    cudaStream_t s = t->s;
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int64_t> pick(0, rows - 1);
    std::vector<int64_t> idx(B);
    std::vector<float> losses(steps, 0.0f);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float b3 = 0;
    cudaMemsetAsync(t->dW0pad, 0, kHid * 16 * 4, s);
    for (int it = 0; it < steps; ++it) {
        for (int b = 0; b < B; ++b) idx[b] = pick(rng);
        cudaMemcpyAsync(t->idx, idx.data(), (size_t)B * 8, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(&b3, t->P + kOffB3, 4, cudaMemcpyDeviceToHost, s);
        cudaMemsetAsync(t->loss, 0, 4, s);
        cudaStreamSynchronize(s);
        k_pack_batch<<<(B + 255) / 256, 256, 0, s>>>(feat, target, t->idx, B, t->fmean, t->fscale, t->X, t->XT,
                                                     t->t);
        cudaError_t e = fwd_bwd(t, b3);
        if (e != cudaSuccess) {
            set_global_error(cudaGetErrorString(e));
            return PBSM3D_ERR_CUDA;
        }
        t->step++;
        const float c1 = 1.0f - powf(b1, (float)t->step), c2 = 1.0f - powf(b2, (float)t->step);
        k_adam<<<64, 256, 0, s>>>(t->P, t->G, t->Mo, t->Vo, kNumParams, lr, b1, b2, eps, c1, c2);
        cudaMemsetAsync(t->dW0pad, 0, kHid * 16 * 4, s);
        refresh_bf16(t);
        cudaMemcpyAsync(&losses[it], t->loss, 4, cudaMemcpyDeviceToHost, s);
    }
    int err = 0;
    cudaMemcpyAsync(&err, t->err, 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || err) {
        set_global_error(err ? "mlp: tensor-core wait timed out" : "mlp: CUDA error in training");
        return PBSM3D_ERR_CUDA;
    }
    if (loss_per_step) std::copy(losses.begin(), losses.end(), loss_per_step);
    return PBSM3D_OK;
}

// C[M][N] (fp32, host) = A[M][K] (bf16 bits) * B[N][K]^T on the tensor cores.
int pbsm3d_mlp_gemm_bf16(const uint16_t* A, const uint16_t* Bm, float* C, int32_t M, int32_t N, int32_t K) {
    if (!A || !Bm || !C || M < 128 || M % 128 || (N != 16 && N != 128) || !(K == 16 || (K >= 64 && K % 64 == 0)))
        return PBSM3D_ERR_INVALID_ARG;
    bf16 *dA = nullptr, *dB = nullptr;
    float* dC = nullptr;
    int* derr = nullptr;
    int rc = PBSM3D_OK;
    if (cudaMalloc(&dA, (size_t)M * K * 2) != cudaSuccess || cudaMalloc(&dB, (size_t)N * K * 2) != cudaSuccess ||
        cudaMalloc(&dC, (size_t)M * N * 4) != cudaSuccess || cudaMalloc(&derr, 4) != cudaSuccess) {
        rc = PBSM3D_ERR_OUT_OF_MEMORY;
    } else {
        cudaMemcpy(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, Bm, (size_t)N * K * 2, cudaMemcpyHostToDevice);
        cudaMemset(derr, 0, 4);
        GemmArgs g{dA, K, dB, K, M, K, K, nullptr, nullptr, 0, nullptr, 0, nullptr, 0, dC, derr};
        cudaError_t e = N == 128 ? launch_gemm<128, EPI_F32>(g, 1, 0) : launch_gemm<16, EPI_F32>(g, 1, 0);
        int err = 0;
        if (e == cudaSuccess) e = cudaMemcpy(C, dC, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(&err, derr, 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess || err) {
            set_global_error(err ? "gemm: tensor-core wait timed out" : cudaGetErrorString(e));
            rc = PBSM3D_ERR_CUDA;
        }
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(derr);
    return rc;
}

}  // extern "C"
