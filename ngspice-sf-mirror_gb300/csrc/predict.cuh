/*
 * Newton predictor inside the transient kernel (engine addition; the
 * reference starts each timestep's Newton iteration from the previous
 * solution with the devices' INITPRED extrapolation, niiter.c:29-367).
 *
 * At each new timestep the unknowns get the linear extrapolation of the
 * last two accepted points, v_n + r1 (v_n - v_{n-1}) with r1 = h_{n+1}/h_n
 * (at most NGSF_PRED_RATIO_MAX), and with a trained network (kind 2) the
 * node voltages add NGSF_PRED_VSCALE times its output.  The network is the
 * message-passing model of gnn.cu run per 128-node tile on the tensor
 * cores of this block: features and aggregated neighbour activations are
 * staged as BF16 core-matrix tiles in shared memory, tcgen05.mma
 * accumulates in tensor memory (FP32), tcgen05.ld brings each row back to
 * its thread for bias, activation and the residual.
 *
 * Included by engine.cu inside its anonymous namespace, after Ctl, Iter
 * and iter_ctx.
 */
#ifndef NGSF_PREDICT_CUH
#define NGSF_PREDICT_CUH

#include "tc05.cuh"

#define PRED_STAGE_BYTES (48 * 1024)   /* A tile 32 KB + B tile 16 KB */

__shared__ uint32_t g_tmem;                    /* 128 accumulator columns */
__shared__ __align__(8) unsigned long long g_pbar;
__shared__ unsigned char *g_psm;               /* staging, or null */
__shared__ uint32_t g_pphase;
__shared__ int g_ptmem;                        /* the block holds tensor memory */

/* kernel start, all threads: tensor memory and the completion barrier for
 * a block that may run a circuit with a trained network (sm: the staging
 * area, null when no circuit of the launch has one) */
__device__ void pred_block_init(unsigned char *sm)
{
    const bool on = sm != nullptr;
    if (threadIdx.x == 0) {
        g_psm = sm;
        g_pphase = 0;
        g_ptmem = on;
        if (on)
            tc05_mbar_init(tc05_smem_u32(&g_pbar), 1);
    }
    if (on && threadIdx.x < 32)
        tc05_tmem_alloc(tc05_smem_u32(&g_tmem), 128);
    tc05_fence_before();
    __syncthreads();
    tc05_fence_after();
}

/* kernel end, all threads */
__device__ void pred_block_fini()
{
    tc05_fence_before();
    __syncthreads();
    if (g_ptmem && threadIdx.x < 32)
        tc05_tmem_dealloc(g_tmem, 128);
}

/* a point was accepted: shift the history (all threads) */
__device__ void pred_accept(const ngsf_ckt_t &C, Ctl &s)
{
    const ngsf_pred_t &P = C.pred;
    if (!P.kind)
        return;
    Iter it = iter_ctx(C, s);
    for (int k = threadIdx.x; k <= C.n; k += blockDim.x) {
        P.h1[k] = P.h0[k];
        P.h0[k] = P.cur[k];
        P.cur[k] = it.rhsOld[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s.th1 = s.th0;
        s.th0 = s.tcur;
        s.tcur = s.time;
        s.histCount++;
        s.guessOff = 0;
    }
    __syncthreads();
}

/* one product on the staged tiles: kt/16 MMAs of M=128, N=n, K=16, then
 * wait for completion (bounded).  All threads call; false on timeout. */
__device__ bool pred_mma(int n, int kt)
{
    const uint32_t sa = tc05_smem_u32(g_psm), sb = sa + 32768;
    const uint32_t bar = tc05_smem_u32(&g_pbar);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc05_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc05_fence_after();
        const uint32_t sbo = (uint32_t)(kt / 8) * 128, idesc = tc05_instr_desc(n);
        for (int q = 0; q < kt / 16; q++)
            tc05_mma_bf16(g_tmem, tc05_smem_desc(sa + q * 256, 128, sbo),
                          tc05_smem_desc(sb + q * 256, 128, sbo), idesc, q ? 1u : 0u);
        tc05_commit(bar);
    }
    /* every thread waits on its own count: the block agrees on the
     * outcome, so all threads leave the product loops together */
    const bool ok = __syncthreads_and(tc05_mbar_wait(bar, g_pphase) ? 1 : 0) != 0;
    if (!ok) {
        /* the committed products may still be running: wait for them once
         * more (bounded) before anything reuses the staging or the tensor
         * memory; if they still have not finished, the network stays off
         * for the rest of the launch (the plain start is used) */
        const bool late = __syncthreads_and(tc05_mbar_wait(bar, g_pphase) ? 1 : 0) != 0;
        if (!late && threadIdx.x == 0)
            g_psm = nullptr;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        g_pphase ^= 1u;
    tc05_fence_after();
    return ok;
}

__device__ __forceinline__ unsigned short bf16_bits(float f)
{
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}

/* 8 consecutive floats -> 8 bf16 into the staged tile (16 bytes) */
__device__ __forceinline__ void put8(unsigned char *tile, int r, int k, int kt, const float *v)
{
    uint4 u;
    u.x = bf16_bits(v[0]) | ((uint32_t)bf16_bits(v[1]) << 16);
    u.y = bf16_bits(v[2]) | ((uint32_t)bf16_bits(v[3]) << 16);
    u.z = bf16_bits(v[4]) | ((uint32_t)bf16_bits(v[5]) << 16);
    u.w = bf16_bits(v[6]) | ((uint32_t)bf16_bits(v[7]) << 16);
    *(uint4 *)(tile + tc05_off(r, k, kt)) = u;
}

/* The network over every voltage node; adds the correction to rhsOld,
 * which already holds the linear extrapolation.  All threads call;
 * warps 0-3 read accumulator lanes 32w..32w+31.  false on a timeout. */
__device__ bool pred_network(const ngsf_ckt_t &C, const Iter &it, double r1, double r2)
{
    const ngsf_pred_t &P = C.pred;
    const int nv = P.nv, nt = (nv + 127) / 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *sA = g_psm, *sB = g_psm + 32768;
    const double VS = NGSF_PRED_VSCALE;
    bool ok = true;

    /* encoder: X [128 x 16] . WinT [64 x 16]^T */
    tc05_stage_tile(sB, P.WinT, 16, 0, 64, 64, 0, 16);
    for (int t = 0; t < nt && ok; t++) {
        for (int c = threadIdx.x; c < 256; c += blockDim.x) {
            const int r = c >> 1, g = c & 1, v = t * 128 + r;
            float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (v < nv) {
                const int k = P.vnode[v];
                const double v3 = P.cur[k], v2 = P.h0[k], v1 = P.h1[k];
                const double d1 = v3 - v2;
                if (g == 0) {
                    f[0] = (float)v3;
                    f[1] = (float)(d1 / VS);
                    f[2] = (float)((v2 - v1) / VS);
                    f[3] = (float)r1;
                    f[4] = (float)r2;
                    f[5] = (float)(r1 * d1 / VS);
                    f[6] = P.stat[(size_t)v * 6 + 0];
                    f[7] = P.stat[(size_t)v * 6 + 1];
                } else {
                    f[0] = P.stat[(size_t)v * 6 + 2];
                    f[1] = P.stat[(size_t)v * 6 + 3];
                    f[2] = P.stat[(size_t)v * 6 + 4];
                    f[3] = P.stat[(size_t)v * 6 + 5];
                    f[4] = 1.0f;
                    /* quadratic-extrapolation increment through the last
                     * three points, beyond the linear one */
                    f[5] = (float)(r1 * (r1 + 1.0) * r2 * (d1 - r2 * (v2 - v1)) / ((r2 + 1.0) * VS));
                }
            }
            put8(sA, r, g * 8, 16, f);
        }
        ok = pred_mma(64, 16);
        if (ok && warp < 4) {
            const int v = t * 128 + warp * 32 + lane;
            for (int c0 = 0; c0 < 64; c0 += 16) {
                float a[16];
                tc05_ld16(g_tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, a);
                if (v < nv)
                    for (int j = 0; j < 16; j++) {
                        const float z = a[j] + P.bin[c0 + j];
                        P.Ha[(size_t)v * 64 + c0 + j] = z > 0.f ? z : 0.f;
                    }
            }
        }
        tc05_fence_before();
        __syncthreads();
    }

    /* three layers: [H | mean of neighbours' H] [128 x 128] . WT [64 x 128]^T */
    for (int l = 0; l < 3 && ok; l++) {
        const float *Hin = (l & 1) ? P.Hb : P.Ha;
        float *Hout = (l & 1) ? P.Ha : P.Hb;
        tc05_stage_tile(sB, P.WT[l], 128, 0, 64, 64, 0, 128);
        for (int t = 0; t < nt && ok; t++) {
            for (int c = threadIdx.x; c < 128 * 16; c += blockDim.x) {
                const int r = c >> 4, g = c & 15, v = t * 128 + r;
                float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                if (v < nv) {
                    if (g < 8) {
                        const float4 *h = (const float4 *)(Hin + (size_t)v * 64 + g * 8);
                        float4 a = h[0], b = h[1];
                        f[0] = a.x, f[1] = a.y, f[2] = a.z, f[3] = a.w;
                        f[4] = b.x, f[5] = b.y, f[6] = b.z, f[7] = b.w;
                    } else {
                        for (int q = P.gptr[v]; q < P.gptr[v + 1]; q++) {
                            const float4 *h =
                                (const float4 *)(Hin + (size_t)P.gidx[q] * 64 + (g - 8) * 8);
                            float4 a = h[0], b = h[1];
                            f[0] += a.x, f[1] += a.y, f[2] += a.z, f[3] += a.w;
                            f[4] += b.x, f[5] += b.y, f[6] += b.z, f[7] += b.w;
                        }
                        const float di = P.dinv[v];
                        for (int j = 0; j < 8; j++)
                            f[j] *= di;
                    }
                }
                put8(sA, r, g * 8, 128, f);
            }
            ok = pred_mma(64, 128);
            if (ok && warp < 4) {
                const int v = t * 128 + warp * 32 + lane;
                for (int c0 = 0; c0 < 64; c0 += 16) {
                    float a[16];
                    tc05_ld16(g_tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, a);
                    if (v < nv)
                        for (int j = 0; j < 16; j++) {
                            const float z = a[j] + P.bl[l][c0 + j];
                            Hout[(size_t)v * 64 + c0 + j] =
                                (z > 0.f ? z : 0.f) + Hin[(size_t)v * 64 + c0 + j];
                        }
                }
            }
            tc05_fence_before();
            __syncthreads();
        }
    }

    /* decoder: H3 [128 x 64] . WoutT [16 x 64]^T, column 0 */
    const float *H3 = P.Hb;
    tc05_stage_tile(sB, P.WoutT, 64, 0, 16, 16, 0, 64);
    for (int t = 0; t < nt && ok; t++) {
        for (int c = threadIdx.x; c < 128 * 8; c += blockDim.x) {
            const int r = c >> 3, g = c & 7, v = t * 128 + r;
            float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (v < nv) {
                const float4 *h = (const float4 *)(H3 + (size_t)v * 64 + g * 8);
                float4 a = h[0], b = h[1];
                f[0] = a.x, f[1] = a.y, f[2] = a.z, f[3] = a.w;
                f[4] = b.x, f[5] = b.y, f[6] = b.z, f[7] = b.w;
            }
            put8(sA, r, g * 8, 64, f);
        }
        ok = pred_mma(16, 64);
        if (ok && warp < 4) {
            const int v = t * 128 + warp * 32 + lane;
            float a[16];
            tc05_ld16(g_tmem + ((uint32_t)(warp * 32) << 16), a);
            if (v < nv) {
                /* the correction fades out on quiet nodes, where the
                 * linear extrapolation is already exact */
                const int k = P.vnode[v];
                const double act = fabs(P.cur[k] - P.h0[k]) + fabs(P.h0[k] - P.h1[k]);
                const double gate = act / (act + NGSF_PRED_QUIET);
                it.rhsOld[k] += NGSF_PRED_VOUT * gate * (double)(a[0] + P.bout[0]);
            }
        }
        tc05_fence_before();
        __syncthreads();
    }
    return ok;
}

/* The guess for the timestep about to start (all threads): the linear
 * (kind 1) or quadratic (kinds 2 and 3) extrapolation of every unknown
 * through the last accepted points, plus, with kind 2, the network's
 * correction of the node voltages; marks the mode so the first iteration
 * reads it. */
__device__ void pred_guess(const ngsf_ckt_t &C, Ctl &s)
{
    const ngsf_pred_t &P = C.pred;
    const double hn = s.tcur - s.th0, hp = s.th0 - s.th1;
    const double r1 = hn > 0 ? fmin(s.delta / hn, NGSF_PRED_RATIO_MAX) : 1.0;
    const double r2 = hp > 0 ? fmin(hn / hp, NGSF_PRED_RATIO_MAX) : 1.0;
    const bool quad = P.kind >= 2;
    Iter it = iter_ctx(C, s);
    for (int k = threadIdx.x; k <= C.n; k += blockDim.x) {
        const double d1 = P.cur[k] - P.h0[k], d2 = P.h0[k] - P.h1[k];
        double g = P.cur[k] + r1 * d1;
        if (quad)   /* the parabola through the last three points */
            g += r1 * (r1 + 1.0) * r2 * (d1 - r2 * d2) / (r2 + 1.0);
        it.rhsOld[k] = k ? g : 0.0;
    }
    __syncthreads();
    bool ok = true;
    if (P.kind == 2 && g_psm)
        ok = pred_network(C, it, r1, r2);
    if (threadIdx.x == 0) {
        if (!ok)
            s.flag = NGSF_E_WATCHDOG;
        s.mode |= NGSF_MODEGUESS;
        s.guessUsed = 1;
        s.guessSteps++;
    }
    __syncthreads();
}

#endif
