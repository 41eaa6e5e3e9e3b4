/*
 * Learned Newton predictor: the message-passing network's training and
 * inference kernels.
 *
 * The reference simulator has no learned predictor (its Newton initial
 * guess is the previous solution plus the devices' INITPRED state
 * extrapolation, src/maths/ni/niiter.c:29-367, PREDICTOR undefined); this
 * file is the project's own addition.  Per circuit node the network
 * predicts a correction to the linear extrapolation of the node voltage to
 * the next timepoint:
 *
 *   H0    = relu(X Win + bin)                                X: N x 16
 *   M_l   = D^-1 A H_l                       (mean over graph neighbours)
 *   H_l+1 = relu([H_l | M_l] W_l + b_l) + H_l        l = 0..2, width 64
 *   pred  = (H3 Wout)[:, 0] + bout
 *
 * Every product runs on the tensor cores: tcgen05.mma kind::f16 with BF16
 * operands staged in shared memory (no-swizzle K-major core-matrix layout)
 * and an FP32 accumulator in tensor memory, issued by one thread, completed
 * through an mbarrier and read back with tcgen05.ld.  The backward pass
 * (weight gradients X^T dY split over node ranges, input gradients dY W^T)
 * uses the same kernel.  Aggregation, bias, activation and the optimiser
 * are FP32 CUDA-core kernels.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ngspice_gb300.h"
#include "tc05.cuh"

extern "C" void ngsf_internal_set_error(const char *msg);

namespace {

constexpr int GN_F = 16;       /* input features */
constexpr int GN_H = 64;       /* hidden width */
constexpr int GN_O = 16;       /* decoder width (column 0 is the prediction) */
constexpr int GN_L = 3;        /* message-passing layers */
constexpr int GN_BM = 128;     /* rows per tensor-core tile */
constexpr int GN_BK = 64;      /* K per shared-memory stage */
constexpr int GN_TMEM_COLS = 128;

/* flat parameter layout (FP32 master copy) */
constexpr int P_WIN = 0;                          /* [16][64]  (in, out) */
constexpr int P_BIN = P_WIN + GN_F * GN_H;
constexpr int P_W0 = P_BIN + GN_H;                /* per layer [128][64] + b[64] */
constexpr int P_LSTRIDE = 2 * GN_H * GN_H + GN_H;
constexpr int P_WOUT = P_W0 + GN_L * P_LSTRIDE;   /* [64][16] */
constexpr int P_BOUT = P_WOUT + GN_H * GN_O;
constexpr int P_COUNT = P_BOUT + 1;

/* Copy a rows x kt tile (K-major, bf16, row stride ld elements) into the
 * core-matrix layout: element (r, k) at (r/8)*sbo + (k/8)*128 + (r%8)*16 +
 * (k%8)*2 with sbo = kt/8*128.  16-byte pieces; rows >= nrows are zero. */
__device__ __forceinline__ void stage_tile(unsigned char *dst, const __nv_bfloat16 *src, int ld,
                                           int row0, int nrows, int rows, int k0, int kt)
{
    const int kg = kt / 8, sbo = kg * 128;
    for (int c = threadIdx.x; c < rows * kg; c += blockDim.x) {
        const int r = c / kg, g = c % kg;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (row0 + r < nrows)
            v = *(const uint4 *)(src + (size_t)(row0 + r) * ld + k0 + g * 8);
        *(uint4 *)(dst + (r / 8) * sbo + g * 128 + (r % 8) * 16) = v;
    }
}

/* C[m, n] (+)= sum_k A[m, k] B[n, k]: A [M x K], B [N x K] bf16 K-major
 * (row strides lda, ldb), C FP32 row-major (ldc).  M rows in tiles of 128
 * (grid.x), the K range split over grid.y (atomicAdd into C, which the
 * caller zeroed, when grid.y > 1).  K is a multiple of 16 and of the
 * split; N a multiple of 16, at most 128.  128 threads: warp w reads
 * accumulator lanes 32w..32w+31 (= tile rows). */
__global__ void __launch_bounds__(128)
gnn_gemm_kernel(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, float *Cm,
                int ldc, int M, int N, int K, int kchunk, int *err)
{
    extern __shared__ __align__(1024) unsigned char gsm[];
    unsigned char *sA = gsm;                        /* 128 x 64 bf16 = 16 KB */
    unsigned char *sB = gsm + GN_BM * GN_BK * 2;    /* 128 x 64 bf16 = 16 KB */
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t taddr_s;
    __shared__ int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * GN_BM;
    const int kb = blockIdx.y * kchunk, ke = min(K, kb + kchunk);
    const uint32_t bar = tc05_smem_u32(&mbar);
    if (threadIdx.x == 0) {
        tc05_mbar_init(bar, 1);
        failed = 0;
    }
    if (warp == 0)
        tc05_tmem_alloc(tc05_smem_u32(&taddr_s), GN_TMEM_COLS);
    tc05_fence_before();
    __syncthreads();
    tc05_fence_after();
    const uint32_t tmem = taddr_s;
    const uint32_t idesc = tc05_instr_desc(N);
    uint32_t phase = 0;
    int issued = 0;             /* thread 0: an MMA was issued */
    const bool any = kb < ke;   /* this block has K work (same for all threads) */
    for (int k0 = kb; k0 < ke; k0 += GN_BK) {
        const int kt = min(GN_BK, ke - k0);
        stage_tile(sA, A, lda, row0, M, GN_BM, k0, kt);
        stage_tile(sB, B, ldb, 0, N, N, k0, kt);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            tc05_fence_after();
            const uint32_t sbo = (uint32_t)(kt / 8) * 128;
            for (int s = 0; s < kt / 16; s++) {
                uint64_t ad = tc05_smem_desc(tc05_smem_u32(sA) + s * 256, 128, sbo);
                uint64_t bd = tc05_smem_desc(tc05_smem_u32(sB) + s * 256, 128, sbo);
                tc05_mma_bf16(tmem, ad, bd, idesc, issued ? 1u : 0u);
                issued = 1;
            }
            tc05_commit(bar);
        }
        __syncthreads();
        if (!tc05_mbar_wait(bar, phase)) {
            atomicExch(&failed, 1);
            if (err)
                atomicExch(err, 1);
        }
        phase ^= 1;
        __syncthreads();
        if (failed)
            break;
    }
    if (failed) {
        /* a wait ran out while the committed products may still be
         * running: wait for them once more (bounded) before the block
         * frees the tensor memory they write; the result is discarded
         * either way (err is set) */
        __syncthreads_and(tc05_mbar_wait(bar, phase ^ 1u) ? 1 : 0);
    }
    tc05_fence_after();
    if (!failed && any) {
        const int r = row0 + warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc05_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (r < M) {
                float *dst = Cm + (size_t)r * ldc + c0;
                if (gridDim.y > 1) {
#pragma unroll
                    for (int i = 0; i < 16; i++)
                        atomicAdd(dst + i, v[i]);
                } else {
#pragma unroll
                    for (int i = 0; i < 16; i++)
                        dst[i] = v[i];
                }
            }
        }
    }
    tc05_fence_before();
    __syncthreads();
    if (warp == 0)
        tc05_tmem_dealloc(tmem, GN_TMEM_COLS);
}

/* ------------------------------------------------------------------ */
/* CUDA-core kernels                                                   */
/* ------------------------------------------------------------------ */
/* out[r, c] = bf16(in[r * ldi + c]) for c < cols, 0 for cols <= c < ldo */
__global__ void gnn_to_bf16(const float *in, int ldi, int cols, int rows, __nv_bfloat16 *out,
                            int ldo, int rowsPad)
{
    const long long total = (long long)rowsPad * ldo;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / ldo), c = (int)(i % ldo);
        float v = (r < rows && c < cols) ? in[(size_t)r * ldi + c] : 0.0f;
        out[i] = __float2bfloat16_rn(v);
    }
}

/* out[c, r] = bf16(in[r * ldi + c]): transpose to [colsPad][rowsPad] */
__global__ void gnn_to_bf16_t(const float *in, int ldi, int cols, int rows, __nv_bfloat16 *out,
                              int colsPad, int rowsPad)
{
    const long long total = (long long)rowsPad * colsPad;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / rowsPad), r = (int)(i % rowsPad);
        float v = (r < rows && c < cols) ? in[(size_t)r * ldi + c] : 0.0f;
        out[i] = __float2bfloat16_rn(v);
    }
}

/* out[c, r] = in[r * ld + c] for bf16 [rows][cols] -> [cols][rows] */
__global__ void gnn_bf16_t(const __nv_bfloat16 *in, int ld, int rows, int cols, __nv_bfloat16 *out)
{
    const long long total = (long long)rows * cols;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / rows), r = (int)(i % rows);
        out[i] = in[(size_t)r * ld + c];
    }
}

/* M[i, :] = dinv[i] * sum over neighbours j of H[j, :]  (64 wide, one warp
 * per node, two features per lane, neighbours in CSR order) */
__global__ void gnn_agg(const float *H, const int *ptr, const int *idx, const float *dinv,
                        float *Mo, int N)
{
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N;
         i += (gridDim.x * blockDim.x) >> 5) {
        float a0 = 0.f, a1 = 0.f;
        for (int q = ptr[i]; q < ptr[i + 1]; q++) {
            const float *h = H + (size_t)idx[q] * GN_H;
            a0 += h[lane];
            a1 += h[lane + 32];
        }
        Mo[(size_t)i * GN_H + lane] = a0 * dinv[i];
        Mo[(size_t)i * GN_H + lane + 32] = a1 * dinv[i];
    }
}

/* adjoint of gnn_agg for a symmetric structure, added into dH */
__global__ void gnn_agg_t_add(const float *dM, int ldm, const int *ptr, const int *idx,
                              const float *dinv, float *dH, int N)
{
    const int lane = threadIdx.x & 31;
    for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < N;
         j += (gridDim.x * blockDim.x) >> 5) {
        float a0 = 0.f, a1 = 0.f;
        for (int q = ptr[j]; q < ptr[j + 1]; q++) {
            const int i = idx[q];
            const float *d = dM + (size_t)i * ldm;
            a0 += d[lane] * dinv[i];
            a1 += d[lane + 32] * dinv[i];
        }
        dH[(size_t)j * GN_H + lane] += a0;
        dH[(size_t)j * GN_H + lane + 32] += a1;
    }
}

/* Z += b; H = relu(Z) (+ Hprev) */
__global__ void gnn_bias_act(float *Z, const float *b, const float *Hprev, float *H, int N)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N * GN_H; i += gridDim.x * blockDim.x) {
        float z = Z[i] + b[i % GN_H];
        Z[i] = z;
        float h = z > 0.f ? z : 0.f;
        if (Hprev)
            h += Hprev[i];
        H[i] = h;
    }
}

/* U = [bf16(H) | bf16(M)]  ([rowsPad][128]) */
__global__ void gnn_concat(const float *H, const float *Mm, int N, __nv_bfloat16 *U, int rowsPad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rowsPad * 2 * GN_H;
         i += gridDim.x * blockDim.x) {
        const int r = i / (2 * GN_H), c = i % (2 * GN_H);
        float v = 0.f;
        if (r < N)
            v = c < GN_H ? H[(size_t)r * GN_H + c] : Mm[(size_t)r * GN_H + c - GN_H];
        U[i] = __float2bfloat16_rn(v);
    }
}

/* pred = out[:, 0] + bout; residual r = pred - y; dOut[:, 0] = w r / W */
__global__ void gnn_head(const float *out, const float *bout, const float *y, const float *w,
                         float wsum, float *pred, float *dOut, float *lossAcc, int N)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        float p = out[(size_t)i * GN_O] + bout[0];
        pred[i] = p;
        if (y) {
            float r = p - y[i];
            for (int c = 0; c < GN_O; c++)
                dOut[(size_t)i * GN_O + c] = 0.f;
            dOut[(size_t)i * GN_O] = w[i] * r / wsum;
            atomicAdd(lossAcc, w[i] * r * r / (2.f * wsum));
        }
    }
}

/* dZ = dH * (Z > 0) */
__global__ void gnn_relu_back(const float *dH, const float *Z, float *dZ, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dZ[i] = Z[i] > 0.f ? dH[i] : 0.f;
}

/* g[c] = sum over rows of X[r, c] (cols <= 64), one thread per column */
__global__ void gnn_colsum(const float *X, int ld, int cols, int rows, float *g)
{
    const int c = threadIdx.x;
    if (c >= cols)
        return;
    float a = 0.f;
    for (int r = 0; r < rows; r++)
        a += X[(size_t)r * ld + c];
    g[c] = a;
}

/* dH = dU[:, :64] + dH  (dU row stride 128) */
__global__ void gnn_add_left(const float *dU, float *dH, int N)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N * GN_H; i += gridDim.x * blockDim.x)
        dH[i] += dU[(size_t)(i / GN_H) * 2 * GN_H + (i % GN_H)];
}

/* Adam on the FP32 master weights */
__global__ void gnn_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1,
                         float b2, float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float mi = b1 * m[i] + (1.f - b1) * g[i];
        float vi = b2 * v[i] + (1.f - b2) * g[i] * g[i];
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace

/* ------------------------------------------------------------------ */
/* host side                                                           */
/* ------------------------------------------------------------------ */
struct ngsf_gnn {
    int n = 0, np = 0;               /* nodes, padded to 128 */
    int *ptr = nullptr, *idx = nullptr;
    float *dinv = nullptr;
    float *P = nullptr, *G = nullptr, *Mo = nullptr, *Vo = nullptr;  /* params, grads, Adam */
    int step = 0;
    /* bf16 weight copies: transposed [out][in] for the forward, as stored
     * [in][out] for the input gradients */
    __nv_bfloat16 *WinT = nullptr, *WT[GN_L] = {}, *Wb[GN_L] = {}, *WoutT = nullptr, *Woutb = nullptr;
    /* activations */
    float *X = nullptr, *Z0 = nullptr, *H[GN_L + 1] = {}, *Z[GN_L] = {}, *Mm = nullptr;
    float *out = nullptr, *pred = nullptr, *y = nullptr, *w = nullptr, *dOut = nullptr;
    float *dH = nullptr, *dZ = nullptr, *dU = nullptr, *gtmp = nullptr, *loss = nullptr;
    __nv_bfloat16 *Xb = nullptr, *U[GN_L] = {}, *Hb = nullptr, *Ab = nullptr, *Bb = nullptr;
    int *err = nullptr;
    std::vector<void *> allocs;
};

namespace {

template <class T>
T *dalloc(ngsf_gnn *g, size_t count, std::string &e)
{
    void *p = nullptr;
    if (e.empty()) {
        cudaError_t r = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (r != cudaSuccess) {
            e = std::string("cudaMalloc: ") + cudaGetErrorString(r);
            return nullptr;
        }
        cudaMemset(p, 0, std::max<size_t>(count, 1) * sizeof(T));
        g->allocs.push_back(p);
    }
    return (T *)p;
}

int grid_for(long long n) { return (int)std::min<long long>(4096, (n + 255) / 256 + 1); }

cudaError_t gemm(ngsf_gnn *g, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb,
                 float *C, int ldc, int M, int N, int K, int splits)
{
    static bool attr = false;
    const int smem = 2 * GN_BM * GN_BK * 2;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(gnn_gemm_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess)
            return e;
        attr = true;
    }
    int kchunk = K;
    if (splits > 1) {
        kchunk = (K + splits - 1) / splits;
        kchunk = (kchunk + GN_BK - 1) / GN_BK * GN_BK;
        splits = (K + kchunk - 1) / kchunk;
        cudaMemset(C, 0, (size_t)M * ldc * sizeof(float));
    }
    dim3 grid((M + GN_BM - 1) / GN_BM, splits);
    gnn_gemm_kernel<<<grid, 128, smem>>>(A, lda, B, ldb, C, ldc, M, N, K, kchunk, g->err);
    return cudaGetLastError();
}

/* bf16 copies of the weights from the FP32 master */
cudaError_t refresh_weights(ngsf_gnn *g)
{
    const float *P = g->P;
    gnn_to_bf16_t<<<grid_for(GN_F * GN_H), 256>>>(P + P_WIN, GN_H, GN_H, GN_F, g->WinT, GN_H, GN_F);
    for (int l = 0; l < GN_L; l++) {
        const float *W = P + P_W0 + l * P_LSTRIDE;
        gnn_to_bf16_t<<<grid_for(2 * GN_H * GN_H), 256>>>(W, GN_H, GN_H, 2 * GN_H, g->WT[l], GN_H,
                                                            2 * GN_H);
        gnn_to_bf16<<<grid_for(2 * GN_H * GN_H), 256>>>(W, GN_H, GN_H, 2 * GN_H, g->Wb[l], GN_H,
                                                          2 * GN_H);
    }
    gnn_to_bf16_t<<<grid_for(GN_H * GN_O), 256>>>(P + P_WOUT, GN_O, GN_O, GN_H, g->WoutT, GN_O, GN_H);
    gnn_to_bf16<<<grid_for(GN_H * GN_O), 256>>>(P + P_WOUT, GN_O, GN_O, GN_H, g->Woutb, GN_O, GN_H);
    return cudaGetLastError();
}

#define GCK(x)                                                      \
    do {                                                            \
        cudaError_t e_ = (x);                                       \
        if (e_ != cudaSuccess) {                                    \
            ngsf_internal_set_error(cudaGetErrorString(e_));        \
            return -1;                                              \
        }                                                           \
    } while (0)

int forward(ngsf_gnn *g, const float *Xh)
{
    const int N = g->n, NP = g->np;
    GCK(cudaMemcpy(g->X, Xh, (size_t)N * GN_F * sizeof(float), cudaMemcpyHostToDevice));
    GCK(refresh_weights(g));
    gnn_to_bf16<<<grid_for((long long)NP * GN_F), 256>>>(g->X, GN_F, GN_F, N, g->Xb, GN_F, NP);
    GCK(gemm(g, g->Xb, GN_F, g->WinT, GN_F, g->Z0, GN_H, NP, GN_H, GN_F, 1));
    gnn_bias_act<<<grid_for((long long)N * GN_H), 256>>>(g->Z0, g->P + P_BIN, nullptr, g->H[0], N);
    for (int l = 0; l < GN_L; l++) {
        gnn_agg<<<grid_for((long long)N * 32), 256>>>(g->H[l], g->ptr, g->idx, g->dinv, g->Mm, N);
        gnn_concat<<<grid_for((long long)NP * 2 * GN_H), 256>>>(g->H[l], g->Mm, N, g->U[l], NP);
        GCK(gemm(g, g->U[l], 2 * GN_H, g->WT[l], 2 * GN_H, g->Z[l], GN_H, NP, GN_H, 2 * GN_H, 1));
        gnn_bias_act<<<grid_for((long long)N * GN_H), 256>>>(
            g->Z[l], g->P + P_W0 + l * P_LSTRIDE + 2 * GN_H * GN_H, g->H[l], g->H[l + 1], N);
    }
    gnn_to_bf16<<<grid_for((long long)NP * GN_H), 256>>>(g->H[GN_L], GN_H, GN_H, N, g->Hb, GN_H, NP);
    GCK(gemm(g, g->Hb, GN_H, g->WoutT, GN_H, g->out, GN_O, NP, GN_O, GN_H, 1));
    GCK(cudaGetLastError());
    return 0;
}

int split_for(int np) { return std::max(1, std::min(64, np / 1024)); }

int backward(ngsf_gnn *g)
{
    const int N = g->n, NP = g->np;
    float *G = g->G;
    const int sp = split_for(NP);
    /* decoder: dWout = H3^T dOut (A = H3^T rows 0..63 of 128), dH3 = dOut Wout^T */
    gnn_colsum<<<1, 64>>>(g->dOut, GN_O, 1, N, G + P_BOUT);
    gnn_to_bf16_t<<<grid_for((long long)NP * GN_BM), 256>>>(g->H[GN_L], GN_H, GN_H, N, g->Ab, GN_BM, NP);
    gnn_to_bf16_t<<<grid_for((long long)NP * GN_O), 256>>>(g->dOut, GN_O, GN_O, N, g->Bb, GN_O, NP);
    GCK(gemm(g, g->Ab, NP, g->Bb, NP, g->gtmp, GN_O, GN_BM, GN_O, NP, sp));
    GCK(cudaMemcpy(G + P_WOUT, g->gtmp, GN_H * GN_O * sizeof(float), cudaMemcpyDeviceToDevice));
    gnn_to_bf16<<<grid_for((long long)NP * GN_O), 256>>>(g->dOut, GN_O, GN_O, N, g->Bb, GN_O, NP);
    GCK(gemm(g, g->Bb, GN_O, g->Woutb, GN_O, g->dH, GN_H, NP, GN_H, GN_O, 1));
    for (int l = GN_L - 1; l >= 0; l--) {
        float *Gl = G + P_W0 + l * P_LSTRIDE;
        gnn_relu_back<<<grid_for((long long)N * GN_H), 256>>>(g->dH, g->Z[l], g->dZ, N * GN_H);
        gnn_colsum<<<1, 64>>>(g->dZ, GN_H, GN_H, N, Gl + 2 * GN_H * GN_H);
        /* dW_l = U^T dZ: A = U^T [128][NP], B = dZ^T [64][NP] */
        gnn_bf16_t<<<grid_for((long long)NP * 2 * GN_H), 256>>>(g->U[l], 2 * GN_H, NP, 2 * GN_H, g->Ab);
        gnn_to_bf16_t<<<grid_for((long long)NP * GN_H), 256>>>(g->dZ, GN_H, GN_H, N, g->Bb, GN_H, NP);
        GCK(gemm(g, g->Ab, NP, g->Bb, NP, Gl, GN_H, 2 * GN_H, GN_H, NP, sp));
        /* dU = dZ W_l^T: A = bf16(dZ) [NP][64], B = W_l [128][64] */
        gnn_to_bf16<<<grid_for((long long)NP * GN_H), 256>>>(g->dZ, GN_H, GN_H, N, g->Hb, GN_H, NP);
        GCK(gemm(g, g->Hb, GN_H, g->Wb[l], GN_H, g->dU, 2 * GN_H, NP, 2 * GN_H, GN_H, 1));
        gnn_add_left<<<grid_for((long long)N * GN_H), 256>>>(g->dU, g->dH, N);
        gnn_agg_t_add<<<grid_for((long long)N * 32), 256>>>(g->dU + GN_H, 2 * GN_H, g->ptr, g->idx,
                                                            g->dinv, g->dH, N);
    }
    /* encoder: dWin = X^T dZ0 (A = X^T rows 0..15 of 128) */
    gnn_relu_back<<<grid_for((long long)N * GN_H), 256>>>(g->dH, g->Z0, g->dZ, N * GN_H);
    gnn_colsum<<<1, 64>>>(g->dZ, GN_H, GN_H, N, G + P_BIN);
    gnn_to_bf16_t<<<grid_for((long long)NP * GN_BM), 256>>>(g->X, GN_F, GN_F, N, g->Ab, GN_BM, NP);
    gnn_to_bf16_t<<<grid_for((long long)NP * GN_H), 256>>>(g->dZ, GN_H, GN_H, N, g->Bb, GN_H, NP);
    GCK(gemm(g, g->Ab, NP, g->Bb, NP, g->gtmp, GN_H, GN_BM, GN_H, NP, sp));
    GCK(cudaMemcpy(G + P_WIN, g->gtmp, GN_F * GN_H * sizeof(float), cudaMemcpyDeviceToDevice));
    GCK(cudaGetLastError());
    return 0;
}

}  // namespace

/* ------------------------------------------------------------------ */
/* C ABI                                                               */
/* ------------------------------------------------------------------ */
extern "C" NGSF_API int ngsf_gnn_param_count(void) { return P_COUNT; }

extern "C" NGSF_API ngsf_gnn *ngsf_gnn_create(int nnodes, const int *nbr_ptr, const int *nbr_idx)
{
    if (nnodes <= 0 || !nbr_ptr || (nbr_ptr[nnodes] > 0 && !nbr_idx)) {
        ngsf_internal_set_error("ngsf_gnn_create: bad graph");
        return nullptr;
    }
    ngsf_gnn *g = new ngsf_gnn;
    g->n = nnodes;
    g->np = (nnodes + GN_BM - 1) / GN_BM * GN_BM;
    const int NP = g->np, E = nbr_ptr[nnodes];
    std::string e;
    g->ptr = dalloc<int>(g, nnodes + 1, e);
    g->idx = dalloc<int>(g, E, e);
    g->dinv = dalloc<float>(g, nnodes, e);
    g->P = dalloc<float>(g, P_COUNT, e);
    g->G = dalloc<float>(g, P_COUNT, e);
    g->Mo = dalloc<float>(g, P_COUNT, e);
    g->Vo = dalloc<float>(g, P_COUNT, e);
    g->WinT = dalloc<__nv_bfloat16>(g, GN_H * GN_F, e);
    for (int l = 0; l < GN_L; l++) {
        g->WT[l] = dalloc<__nv_bfloat16>(g, 2 * GN_H * GN_H, e);
        g->Wb[l] = dalloc<__nv_bfloat16>(g, 2 * GN_H * GN_H, e);
        g->U[l] = dalloc<__nv_bfloat16>(g, (size_t)NP * 2 * GN_H, e);
        g->Z[l] = dalloc<float>(g, (size_t)NP * GN_H, e);
    }
    g->WoutT = dalloc<__nv_bfloat16>(g, GN_O * GN_H, e);
    g->Woutb = dalloc<__nv_bfloat16>(g, GN_H * GN_O, e);
    g->X = dalloc<float>(g, (size_t)NP * GN_F, e);
    g->Z0 = dalloc<float>(g, (size_t)NP * GN_H, e);
    for (int l = 0; l <= GN_L; l++)
        g->H[l] = dalloc<float>(g, (size_t)NP * GN_H, e);
    g->Mm = dalloc<float>(g, (size_t)NP * GN_H, e);
    g->out = dalloc<float>(g, (size_t)NP * GN_O, e);
    g->pred = dalloc<float>(g, NP, e);
    g->y = dalloc<float>(g, NP, e);
    g->w = dalloc<float>(g, NP, e);
    g->dOut = dalloc<float>(g, (size_t)NP * GN_O, e);
    g->dH = dalloc<float>(g, (size_t)NP * GN_H, e);
    g->dZ = dalloc<float>(g, (size_t)NP * GN_H, e);
    g->dU = dalloc<float>(g, (size_t)NP * 2 * GN_H, e);
    g->gtmp = dalloc<float>(g, (size_t)GN_BM * GN_H, e);
    g->loss = dalloc<float>(g, 1, e);
    g->Xb = dalloc<__nv_bfloat16>(g, (size_t)NP * GN_F, e);
    g->Hb = dalloc<__nv_bfloat16>(g, (size_t)NP * GN_H, e);
    g->Ab = dalloc<__nv_bfloat16>(g, (size_t)NP * GN_BM, e);
    g->Bb = dalloc<__nv_bfloat16>(g, (size_t)NP * GN_H, e);
    g->err = dalloc<int>(g, 1, e);
    if (e.empty()) {
        std::vector<float> dinv(nnodes);
        for (int i = 0; i < nnodes; i++) {
            int d = nbr_ptr[i + 1] - nbr_ptr[i];
            dinv[i] = d > 0 ? 1.0f / (float)d : 0.0f;
        }
        cudaError_t r = cudaMemcpy(g->ptr, nbr_ptr, (nnodes + 1) * sizeof(int), cudaMemcpyHostToDevice);
        if (r == cudaSuccess && E > 0)
            r = cudaMemcpy(g->idx, nbr_idx, E * sizeof(int), cudaMemcpyHostToDevice);
        if (r == cudaSuccess)
            r = cudaMemcpy(g->dinv, dinv.data(), nnodes * sizeof(float), cudaMemcpyHostToDevice);
        if (r != cudaSuccess)
            e = cudaGetErrorString(r);
    }
    if (!e.empty()) {
        ngsf_internal_set_error(("ngsf_gnn_create: " + e).c_str());
        for (void *p : g->allocs)
            cudaFree(p);
        delete g;
        return nullptr;
    }
    return g;
}

extern "C" NGSF_API void ngsf_gnn_destroy(ngsf_gnn *g)
{
    if (!g)
        return;
    for (void *p : g->allocs)
        cudaFree(p);
    delete g;
}

extern "C" NGSF_API int ngsf_gnn_set_params(ngsf_gnn *g, const float *flat)
{
    GCK(cudaMemcpy(g->P, flat, P_COUNT * sizeof(float), cudaMemcpyHostToDevice));
    GCK(cudaMemset(g->Mo, 0, P_COUNT * sizeof(float)));
    GCK(cudaMemset(g->Vo, 0, P_COUNT * sizeof(float)));
    g->step = 0;
    return 0;
}

extern "C" NGSF_API int ngsf_gnn_get_params(const ngsf_gnn *g, float *flat)
{
    GCK(cudaMemcpy(flat, g->P, P_COUNT * sizeof(float), cudaMemcpyDeviceToHost));
    return 0;
}

static int check_err(ngsf_gnn *g)
{
    int err = 0;
    GCK(cudaMemcpy(&err, g->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        ngsf_internal_set_error("gnn: a tensor-core completion wait ran out");
        return -1;
    }
    return 0;
}

/* X: host [n][16]; pred: host [n] */
extern "C" NGSF_API int ngsf_gnn_forward(ngsf_gnn *g, const float *X, float *pred)
{
    if (forward(g, X))
        return -1;
    gnn_head<<<grid_for(g->n), 256>>>(g->out, g->P + P_BOUT, nullptr, nullptr, 1.f, g->pred,
                                       nullptr, nullptr, g->n);
    GCK(cudaMemcpy(pred, g->pred, g->n * sizeof(float), cudaMemcpyDeviceToHost));
    return check_err(g);
}

/* One training step on one graph sample: forward, weighted squared-error
 * loss, backward, and (lr > 0) an Adam update.  grads (host, optional)
 * receives the gradient in the flat parameter layout. */
extern "C" NGSF_API int ngsf_gnn_train_step(ngsf_gnn *g, const float *X, const float *y,
                                            const float *w, float lr, float *loss, float *grads)
{
    if (forward(g, X))
        return -1;
    std::vector<float> wh(w, w + g->n);
    float wsum = 0.f;
    for (float v : wh)
        wsum += v;
    if (!(wsum > 0.f)) {
        ngsf_internal_set_error("ngsf_gnn_train_step: weights sum to zero");
        return -1;
    }
    GCK(cudaMemcpy(g->y, y, g->n * sizeof(float), cudaMemcpyHostToDevice));
    GCK(cudaMemcpy(g->w, w, g->n * sizeof(float), cudaMemcpyHostToDevice));
    GCK(cudaMemset(g->loss, 0, sizeof(float)));
    GCK(cudaMemset(g->dOut, 0, (size_t)g->np * GN_O * sizeof(float)));
    gnn_head<<<grid_for(g->n), 256>>>(g->out, g->P + P_BOUT, g->y, g->w, wsum, g->pred, g->dOut,
                                       g->loss, g->n);
    if (backward(g))
        return -1;
    if (loss)
        GCK(cudaMemcpy(loss, g->loss, sizeof(float), cudaMemcpyDeviceToHost));
    if (grads)
        GCK(cudaMemcpy(grads, g->G, P_COUNT * sizeof(float), cudaMemcpyDeviceToHost));
    if (lr > 0.f) {
        g->step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - powf(b1, (float)g->step), c2 = 1.f - powf(b2, (float)g->step);
        gnn_adam<<<grid_for(P_COUNT), 256>>>(g->P, g->G, g->Mo, g->Vo, P_COUNT, lr, b1, b2, 1e-8f,
                                              c1, c2);
        GCK(cudaGetLastError());
    }
    GCK(cudaDeviceSynchronize());
    return check_err(g);
}

/* Plain tensor-core product for tests: C[M][N] = A[M][K] B[N][K]^T with
 * bf16 inputs given as FP32 host arrays (rounded here), FP32 result. */
extern "C" NGSF_API int ngsf_gnn_gemm_test(const float *A, const float *B, float *Cout, int M,
                                           int N, int K, int splits)
{
    if (M <= 0 || N <= 0 || K <= 0 || N % 16 || N > 128 || K % 16 || M % GN_BM) {
        ngsf_internal_set_error("ngsf_gnn_gemm_test: M % 128, N % 16 (<= 128), K % 16 required");
        return -1;
    }
    ngsf_gnn tmp;
    std::string e;
    float *dA32 = dalloc<float>(&tmp, (size_t)M * K, e), *dB32 = dalloc<float>(&tmp, (size_t)N * K, e);
    float *dC = dalloc<float>(&tmp, (size_t)M * N, e);
    __nv_bfloat16 *dA = dalloc<__nv_bfloat16>(&tmp, (size_t)M * K, e);
    __nv_bfloat16 *dB = dalloc<__nv_bfloat16>(&tmp, (size_t)N * K, e);
    tmp.err = dalloc<int>(&tmp, 1, e);
    int rc = 0;
    if (!e.empty()) {
        ngsf_internal_set_error(e.c_str());
        rc = -1;
    }
    cudaError_t r = cudaSuccess;
    if (!rc) {
        r = cudaMemcpy(dA32, A, (size_t)M * K * 4, cudaMemcpyHostToDevice);
        if (r == cudaSuccess)
            r = cudaMemcpy(dB32, B, (size_t)N * K * 4, cudaMemcpyHostToDevice);
        if (r == cudaSuccess) {
            gnn_to_bf16<<<grid_for((long long)M * K), 256>>>(dA32, K, K, M, dA, K, M);
            gnn_to_bf16<<<grid_for((long long)N * K), 256>>>(dB32, K, K, N, dB, K, N);
            r = gemm(&tmp, dA, K, dB, K, dC, N, M, N, K, splits);
        }
        if (r == cudaSuccess)
            r = cudaDeviceSynchronize();
        if (r == cudaSuccess)
            r = cudaMemcpy(Cout, dC, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
        if (r != cudaSuccess) {
            ngsf_internal_set_error(cudaGetErrorString(r));
            rc = -1;
        }
        if (!rc)
            rc = check_err(&tmp);
    }
    for (void *p : tmp.allocs)
        cudaFree(p);
    return rc;
}
