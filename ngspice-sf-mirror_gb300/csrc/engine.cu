/*
 * GPU transient engine: the whole `.tran` of one circuit runs inside one
 * thread block, with no host round trip between time points.
 *
 *   DCtran   (src/spicelib/analysis/dctran.c:67-971, XSPICE variant)
 *     -> CKTop / NIiter  (src/maths/ni/niiter.c:29-367)
 *          -> CKTload     per-device load functions writing stamp slots,
 *                         then a deterministic gather into matrix / rhs
 *          -> SMPluFac    left-looking LU refactor on the fixed pivots
 *          -> SMPsolve    level-scheduled forward / backward substitution
 *          -> NIconvTest  + device convergence tests (block reductions)
 *     -> CKTtrunc / CKTterr   block min-reduction over all charges
 *     -> CKTaccept / CKTsetBreak / CKTclrBreak   breakpoint table
 *
 * Control scalars (time, delta, order, mode, ...) live in shared memory;
 * thread 0 updates them between __syncthreads().  Every loop over
 * instances, equations or matrix entries is strided across the block.
 * A batch of independent circuits is one launch with one block per circuit.
 *
 * All arithmetic is FP64.  Every spin or iteration is bounded: Newton loops
 * by NIiter's iteration limit, the time loop by a step budget
 * (NGSF_E_WATCHDOG), so a kernel always returns with a status word.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <cuda/atomic>
#include <cuda_bf16.h>
#include <mutex>
#include <string>
#include <float.h>
#include <math.h>
#include <string.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/ngspice_gb300.h"
#include "ngsf_types.h"
#include "devsup.cuh"

#define NGSF_THREADS 256
#define NGSF_WARPS (NGSF_THREADS / 32)
/* a matrix cell or rhs entry with more contributions is summed by a warp */
#define NGSF_HEAVY 64
/* largest dynamic shared memory a launch asks for (solve buffers) */
#define NGSF_SOLVE_SMEM_MAX (160 * 1024)

/* This file is compiled in parts, three translation units built in
 * parallel (ptxas takes about a minute on each transient kernel):
 * NGSF_PART 1 the batched transient kernel and its host launchers, 2 the
 * wide (whole-grid) launch, 3 the operator surface, the allocation-free
 * stamps and the probes; without NGSF_PART (0) everything at once.  The
 * device functions are shared by all parts; each part compiles the
 * kernels it defines. */
#ifndef NGSF_PART
#define NGSF_PART 0
#endif
#define NGSF_IN(p) (NGSF_PART == 0 || NGSF_PART == (p))
/* defined in part 1, used by every part */
extern "C" int ngsf_solve_smem_bytes(int n, int tags);
extern "C" int ngsf_pred_smem_bytes(int any);

namespace {

struct Ctl {
    double time, delta, olddelta, newdelta, saveDelta;
    double deltaOld[7];
    double ag[7];
    double redd[NGSF_WARPS];
    int redi[NGSF_WARPS];
    int order, mode, firsttime, iterno, noncon, nbreaks;
    int ring[4];
    int rhsSel;            /* 0: rhs=A, rhsOld=B ; 1: swapped */
    int status, accepted, rejected, numIter, tranIter, timePts, npoints, ncap;
    int badpivot, opiter;
    int flag;
    /* resumable state: where the run stands when the kernel exits for a
     * host re-pivot, and the loop locals it needs to continue */
    int phase, shouldReorder, savedIter, savedNoncon, iters0, reorders;
    long long steps;
    /* Newton predictor: accepted times of cur/h0/h1, accepted points in
     * the history, plain start forced for the retry of this step, the
     * current step started from a guess; counters */
    double tcur, th0, th1;
    int histCount, guessOff, guessUsed, guessSteps, guessFirst, guessFalls;
    double delta0;
    /* CKTop fallbacks: gmin stepping and source stepping (cktop.c) */
    int opPhase, gi, itersBefore;
    double gmin, diagGmin, srcFact, factor, oldGmin, gtarget, startgmin, convFact, raise;
    /* synchronised runs: the sharedsync point the run stopped at (0 none,
     * 1 + the reference's loc), redostep as set by the time loop, and the
     * caller's answer (1: redo the step) */
    int syncLoc, syncRedo, syncReply;
};

/* Per-phase clock record (C.prof, optional): thread 0 of the circuit's
 * block adds the SM clock cycles between two block-wide barriers. */
__device__ __forceinline__ long long prof_t(const ngsf_ckt_t &C)
{
    return C.prof ? clock64() : 0;
}
__device__ __forceinline__ void prof_add(const ngsf_ckt_t &C, int k, long long t0)
{
    if (C.prof && threadIdx.x == 0)
        C.prof[k] += clock64() - t0;
}

/* ---------------------------------------------------------------- */
/* block reductions                                                  */
/* ---------------------------------------------------------------- */
__device__ int block_or(Ctl &s, int v)
{
    unsigned m = __ballot_sync(0xffffffffu, v != 0);
    if ((threadIdx.x & 31) == 0)
        s.redi[threadIdx.x >> 5] = m != 0;
    __syncthreads();
    int r = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++)
        r |= s.redi[w];
    __syncthreads();
    return r;
}

__device__ double block_min(Ctl &s, double v)
{
    for (int o = 16; o > 0; o >>= 1)
        v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0)
        s.redd[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = s.redd[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
        r = fmin(r, s.redd[w]);
    __syncthreads();
    return r;
}

/* AlmostEqualUlps (src/maths/misc/equality.c:27-63): two's-complement
 * lexicographic distance in ulps. */
__device__ bool almost_equal_ulps(double a, double b, int maxUlps)
{
    if (a == b)
        return true;
    long long ai = __double_as_longlong(a);
    if (ai < 0)
        ai = (long long)0x8000000000000000ULL - ai;
    long long bi = __double_as_longlong(b);
    if (bi < 0)
        bi = (long long)0x8000000000000000ULL - bi;
    long long d = ai - bi;
    if (d < 0)
        d = -d;
    return d <= maxUlps;
}

/* ---------------------------------------------------------------- */
/* device support (src/spicelib/devices/devsup.c)                   */
/* ---------------------------------------------------------------- */
__device__ void dev_qmeyer(double vgs, double vgd, double von, double vdsat,
                           double *capgs, double *capgd, double *capgb,
                           double phi, double cox)
{
    const double MAGIC_VDS = 0.025;
    double vgst = vgs - von;
    vdsat = NG_MAX(vdsat, MAGIC_VDS);
    if (vgst <= -phi) {
        *capgb = cox / 2;
        *capgs = 0;
        *capgd = 0;
    } else if (vgst <= -phi / 2) {
        *capgb = -vgst * cox / (2 * phi);
        *capgs = 0;
        *capgd = 0;
    } else if (vgst <= 0) {
        *capgb = -vgst * cox / (2 * phi);
        *capgs = vgst * cox / (1.5 * phi) + cox / 3;
        double vds = vgs - vgd;
        if (vds >= vdsat) {
            *capgd = 0;
        } else {
            double vddif = 2.0 * vdsat - vds;
            double vddif1 = vdsat - vds;
            double vddif2 = vddif * vddif;
            *capgd = *capgs * (1.0 - vdsat * vdsat / vddif2);
            *capgs = *capgs * (1.0 - vddif1 * vddif1 / vddif2);
        }
    } else {
        double vds = vgs - vgd;
        vdsat = NG_MAX(vdsat, MAGIC_VDS);
        if (vdsat <= vds) {
            *capgs = cox / 3;
            *capgd = 0;
            *capgb = 0;
        } else {
            double vddif = 2.0 * vdsat - vds;
            double vddif1 = vdsat - vds;
            double vddif2 = vddif * vddif;
            *capgd = cox * (1.0 - vdsat * vdsat / vddif2) / 3;
            *capgs = cox * (1.0 - vddif1 * vddif1 / vddif2) / 3;
            *capgb = 0;
        }
    }
}

/* NIintegrate (src/maths/ni/niinteg.c:18-80), trapezoidal or Gear; st0..st2
 * are the instance's CKTstate0..2 */
__device__ void ni_integrate(const ngsf_ckt_t &C, const Ctl &s, double *st0, const double *st1,
                             const double *st2, double *geq, double *ceq, double cap, int qcap)
{
    int ccap = qcap + 1;
    st0[ccap] = ni_integ_current(C.opt.method, s.order, s.ag[0], s.ag[1], s.ag[2], st0, st1, st2,
                                 qcap);
    *ceq = st0[ccap] - s.ag[0] * st0[qcap];
    *geq = s.ag[0] * cap;
}

/* ---------------------------------------------------------------- */
/* per-iteration context                                             */
/* ---------------------------------------------------------------- */
struct Iter {
    double *st0, *st1, *st2, *st3;
    double *rhs, *rhsOld;
};

__device__ Iter iter_ctx(const ngsf_ckt_t &C, const Ctl &s)
{
    Iter it;
    it.st0 = C.states + (size_t)s.ring[0] * C.nstates;
    it.st1 = C.states + (size_t)s.ring[1] * C.nstates;
    it.st2 = C.states + (size_t)s.ring[2] * C.nstates;
    it.st3 = C.states + (size_t)s.ring[3] * C.nstates;
    it.rhs = s.rhsSel ? C.rhsOld : C.rhs;
    it.rhsOld = s.rhsSel ? C.rhs : C.rhsOld;
    return it;
}

#include "predict.cuh"

/* ---------------------------------------------------------------- */
/* independent source value at the current time (VSRCload/ISRCload)   */
/* ---------------------------------------------------------------- */
__device__ double src_value(const ngsf_src_t &S, int i, const Ctl &s, const ngsf_opts_t &o)
{
    int mode = s.mode;
    if ((mode & (NGSF_MODEDCOP | NGSF_MODEDCTRANCURVE)) && S.dcgiven[i])
        return S.dc[i];
    double time = (mode & NGSF_MODEDC) ? 0.0 : s.time;
    const double *cf = S.coef + (size_t)i * NGSF_MAX_COEFFS;
    int nc = S.ncoef[i];
    double value = 0.0;
    switch (S.kind[i]) {
    default:
        value = S.dc[i];
        break;
    case WF_PULSE: {
        double V1 = cf[0], V2 = cf[1];
        double TD = nc > 2 ? cf[2] : 0.0;
        double TR = nc > 3 && cf[3] > 0.0 ? cf[3] : o.tstep;
        double TF = nc > 4 && cf[4] > 0.0 ? cf[4] : o.tstep;
        double PW = nc > 5 && cf[5] >= 0.0 ? cf[5] : 0.0;
        double PER = nc > 6 && cf[6] > 0.0 ? cf[6] : TR + TF + PW;
        double PHASE = nc > 7 ? cf[7] : 0.0;
        double tmax = 1e99;
        time -= TD;
        if (PHASE > 0.0)
            tmax = PHASE * PER;
        if (time > tmax) {
            value = V1;
        } else {
            if (time > PER) {
                double basetime = PER * floor(time / PER);
                time -= basetime;
            }
            if (time <= 0 || time >= TR + PW + TF)
                value = V1;
            else if (time >= TR && time <= TR + PW)
                value = V2;
            else if (time > 0 && time < TR)
                value = V1 + (V2 - V1) * (time) / TR;
            else
                value = V2 + (V1 - V2) * (time - (TR + PW)) / TF;
        }
        break;
    }
    case WF_SINE: {
        double PHASE = nc > 5 ? cf[5] : 0.0;
        double phase = PHASE * M_PI / 180.0;
        double VO = cf[0], VA = cf[1];
        double FREQ = nc > 2 && cf[2] != 0.0 ? cf[2] : (1 / o.tstop);
        double TD = nc > 3 ? cf[3] : 0.0;
        double THETA = nc > 4 ? cf[4] : 0.0;
        time -= TD;
        if (time <= 0)
            value = VO + VA * sin(phase);
        else
            value = VO + VA * sin(FREQ * time * 2.0 * M_PI + phase) * exp(-time * THETA);
        break;
    }
    case WF_PWL: {
        if (time <= cf[0]) {
            value = cf[1];
            break;
        }
        double end_time = cf[nc - 2];
        if (time > end_time) {
            value = cf[nc - 1];
            break;
        }
        for (int k = 2; k < nc; k += 2) {
            double itime = cf[k];
            if (itime >= time) {
                time -= cf[k - 2];
                time /= cf[k] - cf[k - 2];
                value = cf[k - 1];
                value += time * (cf[k + 1] - cf[k - 1]);
                break;
            }
        }
        break;
    }
    }
    return value;
}

/* ---------------------------------------------------------------- */
/* device loads                                                      */
/* ---------------------------------------------------------------- */
/* CAPload (src/spicelib/devices/cap/capload.c:15-87) */
__device__ void cap_load(const ngsf_ckt_t &C, const Ctl &s, const Iter &it, int t0, int T)
{
    const ngsf_cap_t &K = C.cap;
    int n = K.n, mode = s.mode;
    if (!(mode & (NGSF_MODETRAN | NGSF_MODETRANOP))) {
        for (int i = t0; i < n; i += T)
            for (int k = 0; k < 6; k++)
                C.stampv[K.stamp0 + k * n + i] = 0.0;
        return;
    }
    bool cond1 = ((mode & NGSF_MODEDC) && (mode & NGSF_MODEINITJCT)) ||
                 ((mode & NGSF_MODEUIC) && (mode & NGSF_MODEINITTRAN));
    for (int i = t0; i < n; i += T) {
        int p = K.node[i], q = K.node[n + i], st = K.st[i];
        double m = K.m[i], cap = K.c[i];
        double vcap = cond1 ? K.ic[i] : it.rhsOld[p] - it.rhsOld[q];
        double g = 0.0, ceqv = 0.0;
        double *sv = C.stampv + K.stamp0 + i;
        if (mode & NGSF_MODETRAN) {
            if ((mode & NGSF_MODEINITPRED) && !(mode & NGSF_MODEGUESS)) {
                it.st0[st] = it.st1[st];
            } else {
                it.st0[st] = cap * vcap;
                if (mode & NGSF_MODEINITTRAN)
                    it.st1[st] = it.st0[st];
            }
            double geq, ceq;
            ni_integrate(C, s, it.st0, it.st1, it.st2, &geq, &ceq, cap, st);
            if (mode & NGSF_MODEINITTRAN)
                it.st1[st + 1] = it.st0[st + 1];
            g = m * geq;
            ceqv = m * ceq;
            sv[0] = g;
            sv[n] = g;
            sv[2 * n] = -g;
            sv[3 * n] = -g;
            sv[4 * n] = -ceqv;
            sv[5 * n] = ceqv;
        } else {
            it.st0[st] = cap * vcap;
            for (int k = 0; k < 6; k++)
                sv[k * n] = 0.0;
        }
    }
}

/* RESload (src/spicelib/devices/res/resload.c:15-40) */
__device__ void res_load(const ngsf_ckt_t &C, int t0, int T)
{
    const ngsf_res_t &K = C.res;
    int n = K.n;
    for (int i = t0; i < n; i += T) {
        double g = K.g[i];
        double *sv = C.stampv + K.stamp0 + i;
        sv[0] = g;
        sv[n] = g;
        sv[2 * n] = -g;
        sv[3 * n] = -g;
    }
}

/* VSRCload / ISRCload (vsrc/vsrcload.c, isrc/isrcload.c) */
__device__ void src_load(const ngsf_ckt_t &C, const Ctl &s)
{
    {
        const ngsf_src_t &K = C.vsrc;
        int n = K.n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double *sv = C.stampv + K.stamp0 + i;
            sv[0] = 1.0;
            sv[n] = -1.0;
            sv[2 * n] = 1.0;
            sv[3 * n] = -1.0;
            double value = src_value(K, i, s, C.opt);
            if (s.mode & NGSF_MODETRANOP)
                value *= s.srcFact;
            sv[4 * n] = value;
        }
    }
    {
        const ngsf_src_t &K = C.isrc;
        int n = K.n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double *sv = C.stampv + K.stamp0 + i;
            double value = src_value(K, i, s, C.opt);
            if (s.mode & NGSF_MODETRANOP)
                value *= s.srcFact;
            double m = K.m[i];
            sv[0] = m * value;
            sv[n] = -(m * value);
        }
    }
}

/* MOS1load (src/spicelib/devices/mos1/mos1load.c:17-941), default build:
 * no sensitivity, bypass option 0, PREDICTOR undefined. */
__device__ int mos1_load_one(const ngsf_ckt_t &C, const Ctl &s, const Iter &it, int i)
{
    const ngsf_mos1_t &K = C.mos1;
    const int n = K.n;
    const double *P = K.p;
    double *H = K.h;
#define MP(f) P[(size_t)(f) * n + i]
#define MH(f) H[(size_t)(f) * n + i]
    const int mode = s.mode;
    const int dN = K.node[M1N_D * n + i], gN = K.node[M1N_G * n + i];
    const int bN = K.node[M1N_B * n + i];
    const int dpN = K.node[M1N_DP * n + i], spN = K.node[M1N_SP * n + i];
    (void)dN;
    double *st0 = it.st0 + K.st[i];
    const double *st1 = it.st1 + K.st[i];
    const double *st2 = it.st2 + K.st[i];
    const double type = MP(M1P_TYPE);
    const double vt = MP(M1P_VT);
    const double DrainSatCur = MP(M1P_DSAT), SourceSatCur = MP(M1P_SSAT);
    const double GateSourceOverlapCap = MP(M1P_CGSO);
    const double GateDrainOverlapCap = MP(M1P_CGDO);
    const double GateBulkOverlapCap = MP(M1P_CGBO);
    const double Beta = MP(M1P_BETA), OxideCap = MP(M1P_COX);
    const double gmin = s.gmin;
    const int off = MP(M1P_OFF) != 0.0;
    int Check = 1;
    double xfact = 0.0;
    double vbs, vgs, vds, vbd, vgd, vgb;

    if ((mode & (NGSF_MODEINITFLOAT | NGSF_MODEINITPRED | NGSF_MODEINITSMSIG |
                 NGSF_MODEINITTRAN)) ||
        ((mode & NGSF_MODEINITFIX) && !off)) {
        if (mode & (NGSF_MODEINITPRED | NGSF_MODEINITTRAN)) {
            xfact = s.delta / s.deltaOld[1];
            st0[M1S_VBS] = st1[M1S_VBS];
            vbs = (1 + xfact) * (st1[M1S_VBS]) - (xfact * (st2[M1S_VBS]));
            st0[M1S_VGS] = st1[M1S_VGS];
            vgs = (1 + xfact) * (st1[M1S_VGS]) - (xfact * (st2[M1S_VGS]));
            st0[M1S_VDS] = st1[M1S_VDS];
            vds = (1 + xfact) * (st1[M1S_VDS]) - (xfact * (st2[M1S_VDS]));
            st0[M1S_VBD] = st0[M1S_VBS] - st0[M1S_VDS];
            if (mode & NGSF_MODEGUESS) {
                /* predictor guess: state copies as above, voltages from rhsOld */
                vbs = type * (it.rhsOld[bN] - it.rhsOld[spN]);
                vgs = type * (it.rhsOld[gN] - it.rhsOld[spN]);
                vds = type * (it.rhsOld[dpN] - it.rhsOld[spN]);
            }
        } else {
            vbs = type * (it.rhsOld[bN] - it.rhsOld[spN]);
            vgs = type * (it.rhsOld[gN] - it.rhsOld[spN]);
            vds = type * (it.rhsOld[dpN] - it.rhsOld[spN]);
        }
        vbd = vbs - vds;
        vgd = vgs - vds;
        double vgdo = st0[M1S_VGS] - st0[M1S_VDS];
        double von = type * MH(M1H_VON);
        if (st0[M1S_VDS] >= 0) {
            vgs = dev_fetlim(vgs, st0[M1S_VGS], von);
            vds = vgs - vgd;
            vds = dev_limvds(vds, st0[M1S_VDS]);
            vgd = vgs - vds;
        } else {
            vgd = dev_fetlim(vgd, vgdo, von);
            vds = vgs - vgd;
            vds = -dev_limvds(-vds, -(st0[M1S_VDS]));
            vgs = vgd + vds;
        }
        if (vds >= 0) {
            vbs = dev_pnjlim(vbs, st0[M1S_VBS], vt, MP(M1P_SVCRIT), &Check);
            vbd = vbs - vds;
        } else {
            vbd = dev_pnjlim(vbd, st0[M1S_VBD], vt, MP(M1P_DVCRIT), &Check);
            vbs = vbd + vds;
        }
    } else {
        if ((mode & NGSF_MODEINITJCT) && !off) {
            vds = type * MP(M1P_ICVDS);
            vgs = type * MP(M1P_ICVGS);
            vbs = type * MP(M1P_ICVBS);
            if ((vds == 0) && (vgs == 0) && (vbs == 0) &&
                ((mode & (NGSF_MODETRAN | NGSF_MODEDCOP | NGSF_MODEDCTRANCURVE)) ||
                 (!(mode & NGSF_MODEUIC)))) {
                vbs = -1;
                vgs = type * MP(M1P_TVTO);
                vds = 0;
            }
        } else {
            vbs = vgs = vds = 0;
        }
    }
    vbd = vbs - vds;
    vgd = vgs - vds;
    vgb = vgs - vbs;

    double gbs, cbs, gbd, cbd;
    if (vbs <= -3 * vt) {
        gbs = gmin;
        cbs = gbs * vbs - SourceSatCur;
    } else {
        double evbs = exp(NG_MIN(709.0, vbs / vt));
        gbs = SourceSatCur * evbs / vt + gmin;
        cbs = SourceSatCur * (evbs - 1) + gmin * vbs;
    }
    if (vbd <= -3 * vt) {
        gbd = gmin;
        cbd = gbd * vbd - DrainSatCur;
    } else {
        double evbd = exp(NG_MIN(709.0, vbd / vt));
        gbd = DrainSatCur * evbd / vt + gmin;
        cbd = DrainSatCur * (evbd - 1) + gmin * vbd;
    }
    int dmode = vds >= 0 ? 1 : -1;

    double cdrain, gm, gds, gmbs, von, vdsat;
    {
        double arg, betap, sarg, vgst;
        double vbx = dmode == 1 ? vbs : vbd;
        const double tPhi = MP(M1P_TPHI), gamma = MP(M1P_GAMMA);
        const double lambda = MP(M1P_LAMBDA);
        if (vbx <= 0) {
            sarg = sqrt(tPhi - vbx);
        } else {
            sarg = sqrt(tPhi);
            sarg = sarg - vbx / (sarg + sarg);
            sarg = NG_MAX(0.0, sarg);
        }
        von = (MP(M1P_TVBI) * type) + gamma * sarg;
        vgst = (dmode == 1 ? vgs : vgd) - von;
        vdsat = NG_MAX(vgst, 0.0);
        if (sarg <= 0)
            arg = 0;
        else
            arg = gamma / (sarg + sarg);
        if (vgst <= 0) {
            cdrain = 0;
            gm = 0;
            gds = 0;
            gmbs = 0;
        } else {
            betap = Beta * (1 + lambda * (vds * dmode));
            if (vgst <= (vds * dmode)) {
                cdrain = betap * vgst * vgst * .5;
                gm = betap * vgst;
                gds = lambda * Beta * vgst * vgst * .5;
                gmbs = gm * arg;
            } else {
                cdrain = betap * (vds * dmode) * (vgst - .5 * (vds * dmode));
                gm = betap * (vds * dmode);
                gds = betap * (vgst - (vds * dmode)) +
                      lambda * Beta * (vds * dmode) * (vgst - .5 * (vds * dmode));
                gmbs = gm * arg;
            }
        }
    }
    MH(M1H_VON) = type * von;
    MH(M1H_VDSAT) = type * vdsat;
    double cd = dmode * cdrain - cbd;
    double capbs = MH(M1H_CAPBS), capbd = MH(M1H_CAPBD);

    if (mode & (NGSF_MODETRAN | NGSF_MODETRANOP | NGSF_MODEINITSMSIG)) {
        const double Cbs = MP(M1P_CBS), Cbssw = MP(M1P_CBSSW);
        const double Cbd = MP(M1P_CBD), Cbdsw = MP(M1P_CBDSW);
        const double tDepCap = MP(M1P_TDEPCAP), tBulkPot = MP(M1P_TBULKPOT);
        const double mj = MP(M1P_MJ), mjsw = MP(M1P_MJSW);
        if (Cbs != 0 || Cbssw != 0) {
            if (vbs < tDepCap) {
                const double arg = 1 - vbs / tBulkPot;
                double sarg, sargsw;
                if (mj == mjsw) {
                    if (mj == .5)
                        sarg = sargsw = 1 / sqrt(arg);
                    else
                        sarg = sargsw = exp(-mj * log(arg));
                } else {
                    if (mj == .5)
                        sarg = 1 / sqrt(arg);
                    else
                        sarg = exp(-mj * log(arg));
                    if (mjsw == .5)
                        sargsw = 1 / sqrt(arg);
                    else
                        sargsw = exp(-mjsw * log(arg));
                }
                st0[M1S_QBS] = tBulkPot * (Cbs * (1 - arg * sarg) / (1 - mj) +
                                           Cbssw * (1 - arg * sargsw) / (1 - mjsw));
                capbs = Cbs * sarg + Cbssw * sargsw;
            } else {
                st0[M1S_QBS] = MP(M1P_F4S) + vbs * (MP(M1P_F2S) + vbs * (MP(M1P_F3S) / 2));
                capbs = MP(M1P_F2S) + MP(M1P_F3S) * vbs;
            }
        } else {
            st0[M1S_QBS] = 0;
            capbs = 0;
        }
        if (Cbd != 0 || Cbdsw != 0) {
            if (vbd < tDepCap) {
                const double arg = 1 - vbd / tBulkPot;
                double sarg, sargsw;
                if (mj == .5 && mjsw == .5) {
                    sarg = sargsw = 1 / sqrt(arg);
                } else {
                    if (mj == .5)
                        sarg = 1 / sqrt(arg);
                    else
                        sarg = exp(-mj * log(arg));
                    if (mjsw == .5)
                        sargsw = 1 / sqrt(arg);
                    else
                        sargsw = exp(-mjsw * log(arg));
                }
                st0[M1S_QBD] = tBulkPot * (Cbd * (1 - arg * sarg) / (1 - mj) +
                                           Cbdsw * (1 - arg * sargsw) / (1 - mjsw));
                capbd = Cbd * sarg + Cbdsw * sargsw;
            } else {
                st0[M1S_QBD] = MP(M1P_F4D) + vbd * (MP(M1P_F2D) + vbd * MP(M1P_F3D) / 2);
                capbd = MP(M1P_F2D) + vbd * MP(M1P_F3D);
            }
        } else {
            st0[M1S_QBD] = 0;
            capbd = 0;
        }
        if ((mode & NGSF_MODETRAN) ||
            ((mode & NGSF_MODEINITTRAN) && !(mode & NGSF_MODEUIC))) {
            double geq, ceq;
            ni_integrate(C, s, st0, st1, st2, &geq, &ceq, capbd, M1S_QBD);
            gbd += geq;
            cbd += st0[M1S_CQBD];
            cd -= st0[M1S_CQBD];
            ni_integrate(C, s, st0, st1, st2, &geq, &ceq, capbs, M1S_QBS);
            gbs += geq;
            cbs += st0[M1S_CQBS];
        }
    }
    MH(M1H_CAPBS) = capbs;
    MH(M1H_CAPBD) = capbd;

    int noncon = 0;
    if (!off || !(mode & (NGSF_MODEINITFIX | NGSF_MODEINITSMSIG)))
        if (Check == 1)
            noncon = 1;

    st0[M1S_VBS] = vbs;
    st0[M1S_VBD] = vbd;
    st0[M1S_VGS] = vgs;
    st0[M1S_VDS] = vds;

    double capgs = 0, capgd = 0, capgb = 0;
    if (mode & (NGSF_MODETRAN | NGSF_MODETRANOP | NGSF_MODEINITSMSIG)) {
        const double tPhi = MP(M1P_TPHI);
        if (dmode > 0)
            dev_qmeyer(vgs, vgd, von, vdsat, &st0[M1S_CAPGS], &st0[M1S_CAPGD],
                       &st0[M1S_CAPGB], tPhi, OxideCap);
        else
            dev_qmeyer(vgd, vgs, von, vdsat, &st0[M1S_CAPGD], &st0[M1S_CAPGS],
                       &st0[M1S_CAPGB], tPhi, OxideCap);
        double vgs1 = st1[M1S_VGS];
        double vgd1 = vgs1 - st1[M1S_VDS];
        double vgb1 = vgs1 - st1[M1S_VBS];
        if (mode & (NGSF_MODETRANOP | NGSF_MODEINITSMSIG)) {
            capgs = 2 * st0[M1S_CAPGS] + GateSourceOverlapCap;
            capgd = 2 * st0[M1S_CAPGD] + GateDrainOverlapCap;
            capgb = 2 * st0[M1S_CAPGB] + GateBulkOverlapCap;
        } else {
            capgs = (st0[M1S_CAPGS] + st1[M1S_CAPGS] + GateSourceOverlapCap);
            capgd = (st0[M1S_CAPGD] + st1[M1S_CAPGD] + GateDrainOverlapCap);
            capgb = (st0[M1S_CAPGB] + st1[M1S_CAPGB] + GateBulkOverlapCap);
        }
        if (mode & (NGSF_MODEINITPRED | NGSF_MODEINITTRAN)) {
            st0[M1S_QGS] = (1 + xfact) * st1[M1S_QGS] - xfact * st2[M1S_QGS];
            st0[M1S_QGD] = (1 + xfact) * st1[M1S_QGD] - xfact * st2[M1S_QGD];
            st0[M1S_QGB] = (1 + xfact) * st1[M1S_QGB] - xfact * st2[M1S_QGB];
        } else {
            if (mode & NGSF_MODETRAN) {
                st0[M1S_QGS] = (vgs - vgs1) * capgs + st1[M1S_QGS];
                st0[M1S_QGD] = (vgd - vgd1) * capgd + st1[M1S_QGD];
                st0[M1S_QGB] = (vgb - vgb1) * capgb + st1[M1S_QGB];
            } else {
                st0[M1S_QGS] = vgs * capgs;
                st0[M1S_QGD] = vgd * capgd;
                st0[M1S_QGB] = vgb * capgb;
            }
        }
    }

    double gcgs, ceqgs, gcgd, ceqgd, gcgb, ceqgb;
    if ((mode & NGSF_MODEINITTRAN) || !(mode & NGSF_MODETRAN)) {
        gcgs = ceqgs = gcgd = ceqgd = gcgb = ceqgb = 0;
    } else {
        if (capgs == 0)
            st0[M1S_CQGS] = 0;
        if (capgd == 0)
            st0[M1S_CQGD] = 0;
        if (capgb == 0)
            st0[M1S_CQGB] = 0;
        ni_integrate(C, s, st0, st1, st2, &gcgs, &ceqgs, capgs, M1S_QGS);
        ni_integrate(C, s, st0, st1, st2, &gcgd, &ceqgd, capgd, M1S_QGD);
        ni_integrate(C, s, st0, st1, st2, &gcgb, &ceqgb, capgb, M1S_QGB);
        ceqgs = ceqgs - gcgs * vgs + s.ag[0] * st0[M1S_QGS];
        ceqgd = ceqgd - gcgd * vgd + s.ag[0] * st0[M1S_QGD];
        ceqgb = ceqgb - gcgb * vgb + s.ag[0] * st0[M1S_QGB];
    }

    double ceqbs = type * (cbs - (gbs)*vbs);
    double ceqbd = type * (cbd - (gbd)*vbd);
    double xnrm, xrev, cdreq;
    if (dmode >= 0) {
        xnrm = 1;
        xrev = 0;
        cdreq = type * (cdrain - gds * vds - gm * vgs - gmbs * vbs);
    } else {
        xnrm = 0;
        xrev = 1;
        cdreq = -(type) * (cdrain - gds * (-vds) - gm * vgd - gmbs * vbd);
    }
    const double gdrain = MP(M1P_GDRAIN), gsource = MP(M1P_GSOURCE);
    double *sv = C.stampv + K.stamp0 + i;
    sv[0 * n] = gdrain;
    sv[1 * n] = (gcgd + gcgs + gcgb);
    sv[2 * n] = gsource;
    sv[3 * n] = (gbd + gbs + gcgb);
    sv[4 * n] = (gdrain + gds + gbd + xrev * (gm + gmbs) + gcgd);
    sv[5 * n] = (gsource + gds + gbs + xnrm * (gm + gmbs) + gcgs);
    sv[6 * n] = (-gdrain);
    sv[7 * n] = -gcgb;
    sv[8 * n] = -gcgd;
    sv[9 * n] = -gcgs;
    sv[10 * n] = (-gsource);
    sv[11 * n] = -gcgb;
    sv[12 * n] = -gbd;
    sv[13 * n] = -gbs;
    sv[14 * n] = (-gdrain);
    sv[15 * n] = ((xnrm - xrev) * gm - gcgd);
    sv[16 * n] = (-gbd + (xnrm - xrev) * gmbs);
    sv[17 * n] = (-gds - xnrm * (gm + gmbs));
    sv[18 * n] = (-(xnrm - xrev) * gm - gcgs);
    sv[19 * n] = (-gsource);
    sv[20 * n] = (-gbs - (xnrm - xrev) * gmbs);
    sv[21 * n] = (-gds - xrev * (gm + gmbs));
    sv[22 * n] = -(type * (ceqgs + ceqgb + ceqgd));
    sv[23 * n] = -(ceqbs + ceqbd - type * ceqgb);
    sv[24 * n] = (ceqbd - cdreq + type * ceqgd);
    sv[25 * n] = cdreq + ceqbs + type * ceqgs;

    MH(M1H_MODE) = dmode;
    MH(M1H_CD) = cd;
    MH(M1H_CBS) = cbs;
    MH(M1H_CBD) = cbd;
    MH(M1H_GBS) = gbs;
    MH(M1H_GBD) = gbd;
    MH(M1H_GM) = gm;
    MH(M1H_GDS) = gds;
    MH(M1H_GMBS) = gmbs;
#undef MP
#undef MH
    return noncon;
}

/* MOS1convTest (src/spicelib/devices/mos1/mos1conv.c:13-99) */
__device__ int mos1_conv_one(const ngsf_ckt_t &C, const Iter &it, int i)
{
    const ngsf_mos1_t &K = C.mos1;
    const int n = K.n;
    const double *P = K.p;
    const double *H = K.h;
    const double type = P[(size_t)M1P_TYPE * n + i];
    const int gN = K.node[M1N_G * n + i], bN = K.node[M1N_B * n + i];
    const int dpN = K.node[M1N_DP * n + i], spN = K.node[M1N_SP * n + i];
    const double *st0 = it.st0 + K.st[i];
    double vbs = type * (it.rhs[bN] - it.rhs[spN]);
    double vgs = type * (it.rhs[gN] - it.rhs[spN]);
    double vds = type * (it.rhs[dpN] - it.rhs[spN]);
    double vbd = vbs - vds;
    double vgd = vgs - vds;
    double vgdo = st0[M1S_VGS] - st0[M1S_VDS];
    double delvbs = vbs - st0[M1S_VBS];
    double delvbd = vbd - st0[M1S_VBD];
    double delvgs = vgs - st0[M1S_VGS];
    double delvds = vds - st0[M1S_VDS];
    double delvgd = vgd - vgdo;
#define MH(f) H[(size_t)(f) * n + i]
    double cdhat, cbhat;
    if (MH(M1H_MODE) >= 0)
        cdhat = MH(M1H_CD) - MH(M1H_GBD) * delvbd + MH(M1H_GMBS) * delvbs +
                MH(M1H_GM) * delvgs + MH(M1H_GDS) * delvds;
    else
        cdhat = MH(M1H_CD) - (MH(M1H_GBD) - MH(M1H_GMBS)) * delvbd -
                MH(M1H_GM) * delvgd + MH(M1H_GDS) * delvds;
    cbhat = MH(M1H_CBS) + MH(M1H_CBD) + MH(M1H_GBD) * delvbd + MH(M1H_GBS) * delvbs;
    double tol = C.opt.reltol * NG_MAX(fabs(cdhat), fabs(MH(M1H_CD))) + C.opt.abstol;
    if (fabs(cdhat - MH(M1H_CD)) >= tol)
        return 1;
    tol = C.opt.reltol * NG_MAX(fabs(cbhat), fabs(MH(M1H_CBS) + MH(M1H_CBD))) + C.opt.abstol;
    if (fabs(cbhat - (MH(M1H_CBS) + MH(M1H_CBD))) > tol)
        return 1;
#undef MH
    return 0;
}

#include "bsim4_load.cuh"
#include "dio_eval.cuh"

__device__ int dio_load_one(const ngsf_ckt_t &C, const Ctl &s, const Iter &it, int i)
{
    const ngsf_dio_t &K = C.dio;
    const int n = K.n;
    DevCtx x;
    x.mode = s.mode;
    x.order = s.order;
    x.gmin = s.gmin;
    x.delta = s.delta;
    x.deltaOld1 = s.deltaOld[1];
    x.gear = C.opt.method;
    x.ag0 = s.ag[0];
    x.ag1 = s.ag[1];
    x.ag2 = s.ag[2];
    x.rhsOld = it.rhsOld;
    x.st0 = it.st0;
    x.st1 = const_cast<double *>(it.st1);
    x.st2 = it.st2;
    int node[DIN_COUNT];
    for (int t = 0; t < DIN_COUNT; t++)
        node[t] = K.node[t * n + i];
    return dio_eval(x, K.p + i, (size_t)n, node, K.st[i], C.stampv + K.stamp0 + i, (size_t)n);
}

__device__ int bsim4_load_one(const ngsf_ckt_t &C, const Ctl &s, const Iter &it, int i)
{
    const ngsf_bsim4_t &K = C.bsim4;
    const int n = K.n;
    B4Ctx x;
    x.mode = s.mode;
    x.order = s.order;
    x.gmin = s.gmin;
    x.delta = s.delta;
    x.deltaOld1 = s.deltaOld[1];
    x.gear = C.opt.method;
    x.ag0 = s.ag[0];
    x.ag1 = s.ag[1];
    x.ag2 = s.ag[2];
    x.rhsOld = it.rhsOld;
    x.st0 = it.st0;
    x.st1 = const_cast<double *>(it.st1);
    x.st2 = it.st2;
    int node[B4N_COUNT];
    for (int t = 0; t < B4N_COUNT; t++)
        node[t] = K.node[t * n + i];
    return bsim4_eval(x, K.p + i, (size_t)n, K.h + i, (size_t)n, node, K.st[i],
                      C.stampv + K.stamp0 + i, (size_t)n);
}

/* ---------------------------------------------------------------- */
/* wide launch: hand-over between block 0 and the worker blocks        */
/* ---------------------------------------------------------------- */
#define NGSF_WIDE_SPIN_LIMIT (1LL << 26)   /* polls: a few seconds */

/* grid (and refactor-group) barriers this block has passed in the launch */
__shared__ unsigned long long g_barGen, g_fbarGen;

/* Barrier over nb blocks of a wide launch (every member calls the same
 * sequence of barriers on the same words); with nb == 1 a block barrier.
 * Arrivals count up in one 64-bit word; the block that completes
 * generation g publishes g in a second word, which the others poll (so the
 * polls do not contend with the arrivals).  The wait is bounded and gives
 * up at once after any block's wait ran out (err). */
__device__ void bar_sync(const ngsf_ckt_t &C, int nb, unsigned long long *arrive,
                         unsigned long long *done, unsigned long long &passed)
{
    __syncthreads();
    if (nb <= 1)
        return;
    if (threadIdx.x == 0) {
        const unsigned long long g = passed + 1;
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> bar(*arrive);
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> gen(*done);
        cuda::atomic_ref<int, cuda::thread_scope_device> err(C.wide->err);
        __threadfence();
        const unsigned long long old = bar.fetch_add(1ull, cuda::memory_order_acq_rel);
        if (old + 1 == g * (unsigned long long)nb) {
            gen.store(g, cuda::memory_order_release);
        } else {
            long long spins = 0;
            while (gen.load(cuda::memory_order_acquire) < g) {
                if (++spins > NGSF_WIDE_SPIN_LIMIT || err.load(cuda::memory_order_relaxed)) {
                    err.store(1);
                    break;
                }
            }
        }
        __threadfence();
        passed = g;
    }
    __syncthreads();
}

__device__ void grid_sync(const ngsf_ckt_t &C, int nb)
{
    if (nb <= 1) {
        __syncthreads();
        return;
    }
    bar_sync(C, nb, &C.wide->bar, &C.wide->gen, g_barGen);
}

/* block 0: publish the control words and a command (thread 0 only) */
__device__ void wide_issue(const ngsf_ckt_t &C, const Ctl &s, int cmd)
{
    ngsf_wide_t *w = C.wide;
    w->done = 0;
    w->noncon = 0;
    w->bad = 0;
    w->tmin = (unsigned long long)__double_as_longlong(1e300);
    const unsigned long long *src = (const unsigned long long *)&s;
    for (int k = 0; k < (int)((sizeof(Ctl) + 7) / 8); k++)
        w->ctl[k] = src[k];
    w->cmd = cmd;
    cuda::atomic_ref<int, cuda::thread_scope_device> seq(w->seq);
    seq.fetch_add(1, cuda::memory_order_release);
}

/* Sum of the contributions to every matrix cell and rhs row.  Cells with
 * up to NGSF_HEAVY contributions are summed by one thread in the
 * reference's load order (bit-identical to CKTload).  The few that collect
 * thousands (a supply node's diagonal) are cut into chunks of NGSF_HCHUNK
 * contributions: one warp per chunk, lane-strided partial sums in load
 * order and a fixed butterfly, then the chunk sums in chunk order
 * (gather_heavy_combine).  The rounding then differs from the sequential
 * sum by far less than the 1e-12 stamp tolerance, and is the same for any
 * number of blocks.  Thread t of T, warp gw of GW. */
__device__ void gather(const ngsf_ckt_t &C, const Iter &it, int t, int T, int gw, int GW)
{
    for (int p = t; p < C.nnz; p += T) {
        const int q0 = C.gptr[p], q1 = C.gptr[p + 1];
        if (q1 - q0 > NGSF_HEAVY)
            continue;
        double acc = 0.0;
        for (int q = q0; q < q1; q++)
            acc += C.stampv[C.gsrc[q]];
        C.ax[p] = acc;
    }
    for (int r = t; r <= C.n; r += T) {
        const int q0 = C.rptr[r], q1 = C.rptr[r + 1];
        if (q1 - q0 > NGSF_HEAVY)
            continue;
        double acc = 0.0;
        for (int q = q0; q < q1; q++)
            acc += C.stampv[C.rsrc[q]];
        it.rhs[r] = acc;
    }
    const int lane = threadIdx.x & 31;
    for (int c = gw; c < C.nhchunk; c += GW) {
        const int h = C.hch_cell[c];
        const int p = C.heavy[h];
        const bool isrhs = p < 0;
        const int e = isrhs ? -p - 1 : p;
        const int *ptr = isrhs ? C.rptr : C.gptr;
        const int *src = isrhs ? C.rsrc : C.gsrc;
        const int q0 = ptr[e] + (c - C.hch_ptr[h]) * NGSF_HCHUNK;
        const int q1 = min(ptr[e + 1], q0 + NGSF_HCHUNK);
        double acc = 0.0;
        for (int q = q0 + lane; q < q1; q += 32)
            acc += C.stampv[src[q]];
        for (int o = 16; o > 0; o >>= 1)
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0)
            C.hpart[c] = acc;
    }
}

/* one block, after every chunk sum is visible */
__device__ void gather_heavy_combine(const ngsf_ckt_t &C, const Iter &it)
{
    for (int h = threadIdx.x; h < C.nheavy; h += blockDim.x) {
        double acc = 0.0;
        for (int c = C.hch_ptr[h]; c < C.hch_ptr[h + 1]; c++)
            acc += C.hpart[c];
        const int p = C.heavy[h];
        if (p < 0)
            it.rhs[-p - 1] = acc;
        else
            C.ax[p] = acc;
    }
}

/* The device loads and the gather of one CKTload, shared by nb blocks
 * (this is block b): every instance to one thread of the grid, then the
 * cell sums.  Block 0 (master) also loads the sources.  Ends after a grid
 * barrier; the heavy chunk sums still need gather_heavy_combine.  Returns
 * this block's convergence flag; the others' are ORed into wide->noncon. */
__device__ int load_phase(const ngsf_ckt_t &C, Ctl &s, const Iter &it, int b, int nb, bool master)
{
    const int t = b * blockDim.x + threadIdx.x, T = nb * blockDim.x;
    const long long t0 = master ? prof_t(C) : 0;
    int nc = 0;
    for (int i = t; i < C.bsim4.n; i += T)
        nc |= bsim4_load_one(C, s, it, i);
    cap_load(C, s, it, t, T);
    for (int i = t; i < C.dio.n; i += T)
        nc |= dio_load_one(C, s, it, i);
    for (int i = t; i < C.mos1.n; i += T)
        nc |= mos1_load_one(C, s, it, i);
    res_load(C, t, T);
    if (master)
        src_load(C, s);
    nc = block_or(s, nc);   /* includes __syncthreads: stamps visible */
    if (nb > 1 && threadIdx.x == 0 && nc && !master)
        atomicOr(&C.wide->noncon, 1);
    grid_sync(C, nb);
    if (master)
        prof_add(C, NGSF_P_LOAD, t0);
    const long long t1 = master ? prof_t(C) : 0;
    const int warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    gather(C, it, t, T, b * nw + warp, nb * nw);
    grid_sync(C, nb);
    if (master)
        prof_add(C, NGSF_P_GATHER, t1);
    return nc;
}

__device__ int lu_factor_rl(const ngsf_ckt_t &C, Ctl &s, int b, int nb);
__device__ double trunc_share(const ngsf_ckt_t &C, const Ctl &s, int t0, int T);
__device__ void trunc_publish(const ngsf_ckt_t &C, double t);

/* worker blocks: serve block 0's commands until EXIT (or a timeout) */
__device__ void wide_worker(const ngsf_ckt_t &C, Ctl &s)
{
    ngsf_wide_t *w = C.wide;
    __shared__ int cmd;
    int seen = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            cuda::atomic_ref<int, cuda::thread_scope_device> seq(w->seq);
            long long spins = 0;
            int v;
            while ((v = seq.load(cuda::memory_order_acquire)) == seen) {
                if (++spins > NGSF_WIDE_SPIN_LIMIT)
                    break;
                __nanosleep(128);
            }
            if (v == seen) {
                cuda::atomic_ref<int, cuda::thread_scope_device>(w->err).store(1);
                cmd = NGSF_WIDE_EXIT;
            } else {
                seen = v;
                cmd = w->cmd;
                unsigned long long *dst = (unsigned long long *)&s;
                for (int k = 0; k < (int)((sizeof(Ctl) + 7) / 8); k++)
                    dst[k] = w->ctl[k];
            }
        }
        __syncthreads();
        if (cmd == NGSF_WIDE_EXIT)
            return;
        if (cmd == NGSF_WIDE_LOAD) {
            Iter it = iter_ctx(C, s);
            load_phase(C, s, it, blockIdx.x, gridDim.x, false);
        } else if (cmd == NGSF_WIDE_FACTOR) {
            lu_factor_rl(C, s, blockIdx.x, gridDim.x);
        } else if (cmd == NGSF_WIDE_TRUNC) {
            trunc_publish(C, block_min(s, trunc_share(C, s, blockIdx.x * blockDim.x + threadIdx.x,
                                                      gridDim.x * blockDim.x)));
            grid_sync(C, gridDim.x);
        }
        __syncthreads();
    }
}

/* CKTload: zero, device loads, gather into matrix and rhs; in a wide
 * launch the worker blocks take their share of both. */
__device__ int ckt_load(const ngsf_ckt_t &C, Ctl &s, const Iter &it)
{
    const int nb = C.wide ? gridDim.x : 1;
    if (C.wide && threadIdx.x == 0)
        wide_issue(C, s, NGSF_WIDE_LOAD);
    int nc = load_phase(C, s, it, 0, nb, true);
    gather_heavy_combine(C, it);
    __shared__ int wide_nc;
    if (threadIdx.x == 0) {
        wide_nc = 0;
        if (C.wide) {
            wide_nc = *(volatile int *)&C.wide->noncon;
            if (*(volatile int *)&C.wide->err)
                s.flag = NGSF_E_WATCHDOG;
        }
    }
    __syncthreads();
    return nc | wide_nc;
}

/* SMPluFac: left-looking refactorization on the fixed pivot sequence.
 * One warp per column; columns of one level are independent.
 * Returns 1 when a pivot is zero or not finite, or an L entry is not
 * finite: the host then chooses new pivots from this matrix (the reference
 * re-factors with pivoting when refactoring fails,
 * src/maths/ni/niiter.c:161-195; klu_refactor fails on a zero pivot only,
 * src/maths/KLU/klusmp.c:591-602).  An L entry above a growth limit also
 * asks for new pivots: in the operating point always NGSF_GROWTH (gmin and
 * source stepping move the matrix far from the one the pivots were chosen
 * on), in the transient C.tran_growth when set (off by default: a re-pivot
 * pauses its circuit until the batch's launch ends, and the retry rule of
 * dc_tran catches the pivots that matter). */
#define NGSF_GROWTH 1e6
__device__ __forceinline__ double growth_limit(const ngsf_ckt_t &C, const Ctl &s)
{
    if (s.mode & (NGSF_MODEDCOP | NGSF_MODETRANOP))
        return NGSF_GROWTH;
    return C.tran_growth > 0.0 ? C.tran_growth : DBL_MAX;
}

/* Right-looking refactorization on the fixed pivot sequence, level by
 * level of the column dependency graph.  Level l first checks its pivots
 * and divides the L entries of its pivot columns by their pivots, then
 * every later entry receives the products L(i,k) * U(k,j) of the level's
 * pivots, one thread per destination, products in a fixed order.  The
 * arithmetic is klu_refactor's (src/maths/KLU/klu_refactor.c): a quotient
 * per L entry and an unfused multiply and subtract per product.  Pivot
 * inverses in the L scaling and fused products were tried: on a few
 * matrices whose pivots grow by more than 1e6 in the transient that
 * rounding let Newton fail where klu's arithmetic converges, so the
 * inverse (one per pivot, by the thread that writes the pivot's last
 * update, or at the start when nothing updates it) serves only the
 * backward solve.  The packed descriptors (sc_pk, ud_pk) carry every
 * index an entry needs in one load, and each thread keeps NGSF_RL_ILP
 * entries' loads in flight before it stores: within a level no
 * destination is read by another entry of the level, so the reordering
 * changes no value. */
#define NGSF_RL_SMALL 1024
#define NGSF_RL_ILP 4
__device__ __forceinline__ int rl_level_work(const ngsf_ckt_t &C, int l)
{
    return C.ud_ptr[l + 1] - C.ud_ptr[l] + C.sc_ptr[l + 1] - C.sc_ptr[l];
}

/* level l, first half (threads t of T): pivot checks, L(:,k) /= U(k,k) */
__device__ __forceinline__ int rl_scale(const ngsf_ckt_t &C, double *lux, int l, int t, int T,
                                        double growth)
{
    int bad = 0;
    for (int c = C.rl_ptr[l] + t; c < C.rl_ptr[l + 1]; c += T) {
        double piv = lux[C.cdiag[C.rl_col[c]]];
        if (!(fabs(piv) > 0.0) || !isfinite(piv))
            bad = 1;
    }
    const int e0 = C.sc_ptr[l], e1 = C.sc_ptr[l + 1];
    for (int e = e0 + t; e < e1; e += NGSF_RL_ILP * T) {
        int2 q[NGSF_RL_ILP];
        double x[NGSF_RL_ILP], v[NGSF_RL_ILP];
#pragma unroll
        for (int j = 0; j < NGSF_RL_ILP; j++) {
            const int ej = e + j * T;
            q[j] = ej < e1 ? ((const int2 *)C.sc_pk)[ej] : make_int2(-1, 0);
        }
#pragma unroll
        for (int j = 0; j < NGSF_RL_ILP; j++)
            if (q[j].x >= 0) {
                x[j] = lux[q[j].x];
                v[j] = lux[q[j].y];
            }
#pragma unroll
        for (int j = 0; j < NGSF_RL_ILP; j++)
            if (q[j].x >= 0) {
                const double l_ik = x[j] / v[j];
                lux[q[j].x] = l_ik;
                if (!(fabs(l_ik) <= growth))
                    bad = 1;
            }
    }
    return bad;
}

/* level l, second half: the updates (and the inverse of every pivot whose
 * last update this is) */
__device__ __forceinline__ void rl_update(const ngsf_ckt_t &C, double *lux, int l, int t, int T)
{
    const int d0 = C.ud_ptr[l], d1 = C.ud_ptr[l + 1];
    for (int d = d0 + t; d < d1; d += NGSF_RL_ILP * T) {
        int4 q[NGSF_RL_ILP];
        int dst[NGSF_RL_ILP];
        double a[NGSF_RL_ILP], x[NGSF_RL_ILP], y[NGSF_RL_ILP];
#pragma unroll
        for (int j = 0; j < NGSF_RL_ILP; j++) {
            const int dj = d + j * T;
            q[j] = dj < d1 ? ((const int4 *)C.ud_pk)[dj] : make_int4(0, 0, 0, -1);
        }
#pragma unroll
        for (int j = 0; j < NGSF_RL_ILP; j++) {
            dst[j] = q[j].x >= 0 ? q[j].x : -q[j].x - 1;
            if (d + j * T < d1) {
                a[j] = lux[dst[j]];
                x[j] = lux[q[j].y];
                y[j] = lux[q[j].z];
            }
        }
#pragma unroll
        for (int j = 0; j < NGSF_RL_ILP; j++)
            if (d + j * T < d1) {
                double acc = __dsub_rn(a[j], __dmul_rn(x[j], y[j]));
                if (q[j].x < 0) {
                    const int dj = d + j * T;
                    for (int c = C.ud_cptr[dj] + 1; c < C.ud_cptr[dj + 1]; c++)
                        acc = __dsub_rn(acc, __dmul_rn(lux[C.ud_l[c]], lux[C.ud_u[c]]));
                }
                lux[dst[j]] = acc;
                if (q[j].w >= 0)
                    C.uinv[q[j].w] = 1.0 / acc;
            }
    }
}

/* One block: a whole level, two barriers. */
__device__ __forceinline__ int rl_level_block(const ngsf_ckt_t &C, double *lux, int l,
                                              double growth)
{
    const int bad = rl_scale(C, lux, l, threadIdx.x, blockDim.x, growth);
    __syncthreads();
    rl_update(C, lux, l, threadIdx.x, blockDim.x);
    __syncthreads();
    return bad;
}

/* The solve's copy of the factor values in term order (threads t of T). */
__device__ void solve_pack(const ngsf_ckt_t &C, const double *lux, int t, int T)
{
    for (int q = t; q < C.nlterm; q += T)
        C.lval[q] = lux[C.lr_pos[q]];
    for (int q = t; q < C.nuterm; q += T)
        C.uval[q] = lux[C.ur_pos[q]];
}


/* blocks of a wide launch that take part in the refactorization: enough
 * threads for the widest levels, few enough for a cheap barrier */
#define NGSF_RL_BLOCKS 48

__device__ int lu_factor_rl(const ngsf_ckt_t &C, Ctl &s, int b, int nbAll)
{
    int bad = 0;
    const double growth = growth_limit(C, s);
    if (nbAll <= 1) {
        double *lux = C.lux;
        for (int q = threadIdx.x; q < C.nlu; q += blockDim.x)
            lux[q] = 0.0;
        __syncthreads();
        for (int p = threadIdx.x; p < C.nnz; p += blockDim.x)
            lux[C.a_lupos[p]] = C.ax[p];
        __syncthreads();
        if (s.diagGmin != 0.0) {
            /* LoadGmin: gmin on every structural diagonal (klusmp.c:587-589) */
            for (int j = threadIdx.x; j < C.n; j += blockDim.x)
                if (C.a_diag[j] >= 0)
                    lux[C.a_lupos[C.a_diag[j]]] += s.diagGmin;
            __syncthreads();
        }
        for (int k = threadIdx.x; k < C.n; k += blockDim.x)
            C.uinv[k] = 1.0 / lux[C.cdiag[k]];
        __syncthreads();
        for (int l = 0; l < C.rl_levels; l++)
            bad |= rl_level_block(C, lux, l, growth);
        solve_pack(C, lux, threadIdx.x, blockDim.x);
        return block_or(s, bad);
    }
    /* wide launch: a level with little work runs in block 0 alone (two
     * block barriers); a larger one over the refactorization group (two
     * group barriers), after one barrier that publishes block 0's levels */
    const int nb = min(nbAll, C.rl_blocks > 0 ? C.rl_blocks : NGSF_RL_BLOCKS);
    const int smallWork = C.rl_small > 0 ? C.rl_small : NGSF_RL_SMALL;
    if (b < nb) {
        ngsf_wide_t *w = C.wide;
        auto gsync = [&]() { bar_sync(C, nb, &w->fbar, &w->fgen, g_fbarGen); };
        const int t = b * blockDim.x + threadIdx.x, T = nb * blockDim.x;
        for (int q = t; q < C.nlu; q += T)
            C.lux[q] = 0.0;
        gsync();
        for (int p = t; p < C.nnz; p += T)
            C.lux[C.a_lupos[p]] = C.ax[p];
        gsync();
        if (s.diagGmin != 0.0) {
            for (int j = t; j < C.n; j += T)
                if (C.a_diag[j] >= 0)
                    C.lux[C.a_lupos[C.a_diag[j]]] += s.diagGmin;
            gsync();
        }
        for (int k = t; k < C.n; k += T)
            C.uinv[k] = 1.0 / C.lux[C.cdiag[k]];
        gsync();
        bool pending = false;   /* block 0 ran levels since the last group barrier */
        for (int l = 0; l < C.rl_levels; l++) {
            if (rl_level_work(C, l) <= smallWork) {
                if (b == 0)
                    bad |= rl_level_block(C, C.lux, l, growth);
                pending = true;
            } else {
                if (pending)
                    gsync();
                pending = false;
                bad |= rl_scale(C, C.lux, l, t, T, growth);
                gsync();
                rl_update(C, C.lux, l, t, T);
                gsync();
            }
        }
        if (pending)
            gsync();
        solve_pack(C, C.lux, t, T);
    }
    bad = block_or(s, bad);
    if (threadIdx.x == 0 && bad)
        atomicOr(&C.wide->bad, 1);
    grid_sync(C, nbAll);
    __shared__ int allbad;
    if (threadIdx.x == 0)
        allbad = *(volatile int *)&C.wide->bad;
    __syncthreads();
    return allbad;
}

__device__ int lu_factor(const ngsf_ckt_t &C, Ctl &s)
{
    if (C.rl_levels > 0) {
        const int nb = C.wide ? gridDim.x : 1;
        if (C.wide && threadIdx.x == 0)
            wide_issue(C, s, NGSF_WIDE_FACTOR);
        return lu_factor_rl(C, s, 0, nb);
    }
    for (int q = threadIdx.x; q < C.nlu; q += blockDim.x)
        C.lux[q] = 0.0;
    __syncthreads();
    for (int p = threadIdx.x; p < C.nnz; p += blockDim.x)
        C.lux[C.a_lupos[p]] = C.ax[p];
    __syncthreads();
    if (s.diagGmin != 0.0) {
        /* LoadGmin: gmin on every structural diagonal (klusmp.c:587-589) */
        for (int j = threadIdx.x; j < C.n; j += blockDim.x)
            if (C.a_diag[j] >= 0)
                C.lux[C.a_lupos[C.a_diag[j]]] += s.diagGmin;
        __syncthreads();
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const double growth = growth_limit(C, s);
    int bad = 0;
    for (int l = 0; l < C.nlevels; l++) {
        for (int c = C.lvl_ptr[l] + warp; c < C.lvl_ptr[l + 1]; c += nwarps) {
            int k = C.lvl_col[c];
            for (int t = C.kptr[k]; t < C.kptr[k + 1]; t++) {
                double xk = C.lux[C.kpos[t]];
                for (int u = C.kseg[t] + lane; u < C.kseg[t + 1]; u += 32)
                    C.lux[C.upd_dst[u]] -= C.lux[C.upd_src[u]] * xk;
                __syncwarp();
            }
            double piv = C.lux[C.cdiag[k]];
            if (!(fabs(piv) > 0.0) || !isfinite(piv))
                bad = 1;
            for (int q = C.cdiag[k] + 1 + lane; q < C.cend[k]; q += 32) {
                double l_ik = C.lux[q] / piv;
                C.lux[q] = l_ik;
                if (!(fabs(l_ik) <= growth))
                    bad = 1;
            }
            __syncwarp();
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < C.n; k += blockDim.x)
        C.uinv[k] = 1.0 / C.lux[C.cdiag[k]];
    solve_pack(C, C.lux, threadIdx.x, blockDim.x);
    return block_or(s, bad);
}

/* Triangular-solve workspace of this block: n+1 doubles of dynamic shared
 * memory when they fit the launch's allocation, else C.work. */
__shared__ double *g_sw;

/* Row completion tags of the dependency-driven solve (n ints after the
 * solve vector in dynamic shared memory, or null), and the tag of the
 * sweep in progress: a row is done in this sweep when its tag equals it. */
__shared__ int *g_sflag;
__shared__ int g_stag;

__device__ __forceinline__ size_t solve_vec_bytes(int n)
{
    return ((size_t)(n + 1) * sizeof(double) + 127) & ~(size_t)127;
}

__device__ void solve_buffers_init(const ngsf_ckt_t &C, unsigned char *dyn, int dynBytes)
{
    const bool vec = dyn && solve_vec_bytes(C.n) <= (size_t)dynBytes;
    const bool flags = vec && solve_vec_bytes(C.n) + (size_t)C.n * sizeof(int) <= (size_t)dynBytes;
    if (threadIdx.x == 0) {
        g_sw = vec ? (double *)dyn : nullptr;
        g_sflag = flags ? (int *)(dyn + solve_vec_bytes(C.n)) : nullptr;
        g_stag = 0;
    }
    __syncthreads();
    if (flags)
        for (int i = threadIdx.x; i < C.n; i += blockDim.x)
            g_sflag[i] = 0;
    __syncthreads();
}

/* One thread's row of a triangular-solve level: its descriptor, the first
 * NGSF_SOLVE_PF terms (factor value, column) and, for the backward solve,
 * pivot's inverse.  None of these change during a solve, so a row of level l+1
 * is fetched before the barrier that ends level l, and the level itself
 * then waits only on shared-memory reads of w. */
#define NGSF_SOLVE_PF 6
struct SolveRow {
    int row, q0, q1;
    double piv;
    double v[NGSF_SOLVE_PF];
    int c[NGSF_SOLVE_PF];
};

__device__ __forceinline__ void solve_fetch(SolveRow &p, const int4 *desc, int r, int rEnd,
                                            const double *val, const int *col,
                                            const double *uinv, bool back)
{
    p.row = -1;
    if (r < rEnd) {
        const int4 d = desc[r];
        if (d.z - d.y <= 32) {   /* longer rows are reduced by a warp */
            p.row = d.x;
            p.q0 = d.y;
            p.q1 = d.z;
#pragma unroll
            for (int k = 0; k < NGSF_SOLVE_PF; k++)
                if (d.y + k < d.z) {
                    p.v[k] = val[d.y + k];
                    p.c[k] = col[d.y + k];
                }
            if (back)
                p.piv = uinv[d.x];
        }
    }
}

/* w[row] -= the row's terms, in term order, fused (then x 1/pivot) */
__device__ __forceinline__ void solve_apply(const SolveRow &p, double *w, const double *val,
                                            const int *col, bool back)
{
    if (p.row < 0)
        return;
    double acc = w[p.row];
#pragma unroll
    for (int k = 0; k < NGSF_SOLVE_PF; k++)
        if (p.q0 + k < p.q1)
            acc = fma(-p.v[k], w[p.c[k]], acc);
    for (int q = p.q0 + NGSF_SOLVE_PF; q < p.q1; q++)
        acc = fma(-val[q], w[col[q]], acc);
    w[p.row] = back ? acc * p.piv : acc;
}

/* A warp's long row of a solve level (more than 32 terms): each lane's
 * first NGSF_SOLVE_HPF terms of its lane-strided share, fetched before the
 * barrier like SolveRow. */
#define NGSF_SOLVE_HPF 4
struct SolveHeavy {
    int k, q0, q1;
    double v[NGSF_SOLVE_HPF];
    int c[NGSF_SOLVE_HPF];
};

__device__ __forceinline__ void heavy_fetch(SolveHeavy &h, const int *hrow, int hh, int hEnd,
                                            const int *rptr, const double *val,
                                            const int *col, int lane)
{
    h.k = -1;
    if (hh < hEnd) {
        h.k = hrow[hh];
        h.q0 = rptr[h.k];
        h.q1 = rptr[h.k + 1];
#pragma unroll
        for (int j = 0; j < NGSF_SOLVE_HPF; j++) {
            const int q = h.q0 + lane + 32 * j;
            if (q < h.q1) {
                h.v[j] = val[q];
                h.c[j] = col[q];
            }
        }
    }
}

/* the warp's row: lane-strided partial sums in term order, a fixed
 * butterfly, then w[k] -= sum (x 1/pivot) by lane 0 */
__device__ __forceinline__ void heavy_apply(const ngsf_ckt_t &C, const SolveHeavy &h, double *w,
                                            const double *val, const int *col, int lane,
                                            bool back)
{
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < NGSF_SOLVE_HPF; j++) {
        const int q = h.q0 + lane + 32 * j;
        if (q < h.q1)
            acc = fma(h.v[j], w[h.c[j]], acc);
    }
    for (int q = h.q0 + lane + 32 * NGSF_SOLVE_HPF; q < h.q1; q += 32)
        acc = fma(val[q], w[col[q]], acc);
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0)
        w[h.k] = back ? (w[h.k] - acc) * C.uinv[h.k] : w[h.k] - acc;
}

/* One sweep (forward over L, or backward over U with the division by the
 * pivot): per level, rows of up to 32 terms by one thread each, terms in
 * order; longer rows (listed per level in hptr/hrow) by a warp, with
 * lane-strided partial sums and a fixed butterfly.  Each thread's first
 * row and each warp's first long row of the next level are fetched before
 * the barrier. */
__device__ __forceinline__ void solve_sweep(const ngsf_ckt_t &C, double *w, int nlev, const int *lptr,
                            const int4 *desc, const double *val, const int *col,
                            const int *rptr, const int *hptr, const int *hrow, bool back)
{
    const int t = threadIdx.x, T = blockDim.x;
    const int warp = t >> 5, lane = t & 31, nwarps = T >> 5;
    SolveRow p;
    SolveHeavy hv;
    p.row = -1;
    hv.k = -1;
    if (nlev > 0) {
        solve_fetch(p, desc, lptr[0] + t, lptr[1], val, col, C.uinv, back);
        heavy_fetch(hv, hrow, hptr[0] + warp, hptr[1], rptr, val, col, lane);
    }
    for (int l = 0; l < nlev; l++) {
        const int r1 = lptr[l + 1];
        solve_apply(p, w, val, col, back);
        for (int r = lptr[l] + t + T; r < r1; r += T) {
            SolveRow q;
            solve_fetch(q, desc, r, r1, val, col, C.uinv, back);
            solve_apply(q, w, val, col, back);
        }
        if (hv.k >= 0)
            heavy_apply(C, hv, w, val, col, lane, back);
        for (int h = hptr[l] + warp + nwarps; h < hptr[l + 1]; h += nwarps) {
            SolveHeavy q;
            heavy_fetch(q, hrow, h, hptr[l + 1], rptr, val, col, lane);
            heavy_apply(C, q, w, val, col, lane, back);
        }
        if (l + 1 < nlev) {
            solve_fetch(p, desc, r1 + t, lptr[l + 2], val, col, C.uinv, back);
            heavy_fetch(hv, hrow, hptr[l + 1] + warp, hptr[l + 2], rptr, val, col, lane);
        }
        __syncthreads();
    }
}

/* Dependency-driven sweep: the same rows, terms and arithmetic as
 * solve_sweep (so the same bits), without the barriers between levels.
 * Warp 0 takes the long rows (more than 32 terms) in level order, the other
 * warps' threads the short rows, thread by thread in level order; a row
 * waits for the rows its terms read (their tags in shared memory, acquire)
 * and publishes its own (release).  Every worker takes its rows in level
 * order and rows of one level do not read one another, so the earliest
 * unfinished row can always proceed.  A wait is bounded: one that runs out
 * (NGSF_SF_SPIN polls) flags the block and the sweep goes on without it. */
#define NGSF_SF_SPIN (1 << 22)
/* set when a wait of the sweep ran out: every later wait then returns at
 * once, so one stall bounds the whole sweep */
__shared__ int g_sf_abort;

__device__ __forceinline__ bool sf_wait(int *flags, int c, int tag)
{
    cuda::atomic_ref<int, cuda::thread_scope_block> f(flags[c]);
    for (int i = 0; i < NGSF_SF_SPIN; i++) {
        if (f.load(cuda::memory_order_acquire) == tag)
            return true;
        if (*(volatile int *)&g_sf_abort)
            return false;
        if (i >= 32)
            __nanosleep(32);   /* leave the issue slots to the rows it waits for */
    }
    *(volatile int *)&g_sf_abort = 1;
    return false;
}

__device__ __forceinline__ void sf_publish(int *flags, int row, int tag)
{
    cuda::atomic_ref<int, cuda::thread_scope_block> f(flags[row]);
    f.store(tag, cuda::memory_order_release);
}

__device__ int solve_sweep_sf(const ngsf_ckt_t &C, double *w, int *flags, int tag, int nlev,
                              const int *lptr, const int4 *desc, const double *val,
                              const int *col, const int *rptr, const int *hptr,
                              const int *hrow, bool back)
{
    const int t = threadIdx.x, T = blockDim.x;
    const int warp = t >> 5, lane = t & 31;
    int late = 0;
    if (warp == 0) {
        for (int h = hptr[0]; h < hptr[nlev]; h++) {
            const int k = hrow[h];
            const int q0 = rptr[k], q1 = rptr[k + 1];
            double acc = 0.0;
            for (int q = q0 + lane; q < q1; q += 32) {
                const int c = col[q];
                const double v = val[q];
                if (!sf_wait(flags, c, tag))
                    late = 1;
                acc = fma(v, w[c], acc);
            }
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) {
                w[k] = back ? (w[k] - acc) * C.uinv[k] : w[k] - acc;
                sf_publish(flags, k, tag);
            }
            __syncwarp();
        }
    } else {
        for (int r = lptr[0] + t - 32; r < lptr[nlev]; r += T - 32) {
            const int4 d = desc[r];
            if (d.z - d.y > 32)
                continue;
            double acc = w[d.x];
            for (int q = d.y; q < d.z; q++) {
                const int c = col[q];
                const double v = val[q];
                if (!sf_wait(flags, c, tag))
                    late = 1;
                acc = fma(-v, w[c], acc);
            }
            w[d.x] = back ? acc * C.uinv[d.x] : acc;
            sf_publish(flags, d.x, tag);
        }
    }
    __syncthreads();
    return late;
}

/* SMPsolve: x = A^-1 b, in place on rhs (row-oriented; dependency driven
 * when the block has room for the row tags and C.solve_sf is set, else
 * level by level).  Returns nonzero when a bounded wait ran out. */
__device__ int lu_solve(const ngsf_ckt_t &C, Ctl &s, double *rhs)
{
    double *w = g_sw ? g_sw : C.work;
    for (int k = threadIdx.x; k < C.n; k += blockDim.x)
        w[k] = rhs[C.prow[k]];
    __syncthreads();
    int late = 0;
    if (g_sflag && C.solve_sf && blockDim.x > 32) {
        __shared__ int tag;
        if (threadIdx.x == 0) {
            tag = (g_stag += 2);
            g_sf_abort = 0;
        }
        __syncthreads();
        const int tg = tag;
        late |= solve_sweep_sf(C, w, g_sflag, tg - 1, C.nflevels, C.fl_ptr,
                               (const int4 *)C.fdesc, C.lval, C.lr_col, C.lr_ptr, C.fh_ptr,
                               C.fh_row, false);
        late |= solve_sweep_sf(C, w, g_sflag, tg, C.nblevels, C.bl_ptr, (const int4 *)C.bdesc,
                               C.uval, C.ur_col, C.ur_ptr, C.bh_ptr, C.bh_row, true);
        late = block_or(s, late);
    } else {
        solve_sweep(C, w, C.nflevels, C.fl_ptr, (const int4 *)C.fdesc, C.lval, C.lr_col,
                    C.lr_ptr, C.fh_ptr, C.fh_row, false);
        solve_sweep(C, w, C.nblevels, C.bl_ptr, (const int4 *)C.bdesc, C.uval, C.ur_col,
                    C.ur_ptr, C.bh_ptr, C.bh_row, true);
    }
    for (int k = threadIdx.x; k < C.n; k += blockDim.x)
        rhs[C.pcol[k]] = w[k];
    __syncthreads();
    return late;
}

/* NIconvTest (src/maths/ni/niconv.c:21-90).
 * The reference then calls CKTconvTest (cktop.c:126-145), which runs the
 * device current tests (MOS1convTest, ...) but returns their *error code*,
 * always OK; the CKTnoncon those tests increment is overwritten when NIiter
 * stores NIconvTest's return value (niiter.c:286-289).  The device tests
 * therefore never change a Newton decision, and the engine does not spend
 * FP64 work on them (mos1_conv_one stays available for diagnostics). */
__device__ int conv_test(const ngsf_ckt_t &C, Ctl &s, const Iter &it, bool voltagesOnly = false)
{
    int bad = 0;
    for (int i = 1 + threadIdx.x; i <= C.n; i += blockDim.x) {
        if (voltagesOnly && !C.ntype[i])
            continue;
        double nw = it.rhs[i], od = it.rhsOld[i];
        if (isnan(nw)) {
            bad = 1;
            break;
        }
        double tol = C.opt.reltol * NG_MAX(fabs(od), fabs(nw)) +
                     (C.ntype[i] ? C.opt.vntol : C.opt.abstol);
        if (fabs(nw - od) > tol) {
            bad = 1;
            break;
        }
    }
    return block_or(s, bad);
}

/* CKTterr (src/spicelib/analysis/cktterr.c:13-79), trapezoidal or Gear */
__device__ double ckt_terr(const ngsf_ckt_t &C, const Ctl &s, int qcap, double timeStep)
{
    const ngsf_opts_t &o = C.opt;
    const double *st0 = C.states + (size_t)s.ring[0] * C.nstates;
    const double *st1 = C.states + (size_t)s.ring[1] * C.nstates;
    int ccap = qcap + 1;
    double volttol = o.abstol + o.reltol * NG_MAX(fabs(st0[ccap]), fabs(st1[ccap]));
    double chargetol = NG_MAX(fabs(st0[qcap]), fabs(st1[qcap]));
    chargetol = o.reltol * NG_MAX(chargetol, o.chgtol) / s.delta;
    double tol = NG_MAX(volttol, chargetol);
    double diff[8], deltmp[8];
    for (int i = s.order + 1; i >= 0; i--)
        diff[i] = C.states[(size_t)s.ring[i] * C.nstates + qcap];
    for (int i = 0; i <= s.order; i++)
        deltmp[i] = s.deltaOld[i];
    int j = s.order;
    for (;;) {
        for (int i = 0; i <= j; i++)
            diff[i] = (diff[i] - diff[i + 1]) / deltmp[i];
        if (--j < 0)
            break;
        for (int i = 0; i <= j; i++)
            deltmp[i] = deltmp[i + 1] + s.deltaOld[i];
    }
    /* error constants of the methods by order (cktterr.c:28-39) */
    const double trapCoeff[2] = {.5, .08333333333};
    const double gearCoeff[2] = {.5, .2222222222};
    double factor = C.opt.method ? gearCoeff[s.order - 1] : trapCoeff[s.order - 1];
    double del = o.trtol * tol / NG_MAX(o.abstol, factor * fabs(diff[0]));
    if (s.order == 2)
        del = sqrt(del);
    return NG_MIN(timeStep, del);
}

/* DEVtrunc of the charges this thread owns (thread t0 of T): the smallest
 * CKTterr step among them */
__device__ __forceinline__ double trunc_share(const ngsf_ckt_t &C, const Ctl &s, int t0, int T)
{
    double t = 1e300;   /* HUGE */
    for (int i = t0; i < C.cap.n; i += T)
        t = ckt_terr(C, s, C.cap.st[i], t);
    for (int i = t0; i < C.dio.n; i += T)
        t = ckt_terr(C, s, C.dio.st[i] + DIS_CAPCHARGE, t);
    for (int i = t0; i < C.bsim4.n; i += T) {
        int b = C.bsim4.st[i];
        t = ckt_terr(C, s, b + B4S_QB, t);
        t = ckt_terr(C, s, b + B4S_QG, t);
        t = ckt_terr(C, s, b + B4S_QD, t);
    }
    for (int i = t0; i < C.mos1.n; i += T) {
        int b = C.mos1.st[i];
        t = ckt_terr(C, s, b + M1S_QGS, t);
        t = ckt_terr(C, s, b + M1S_QGD, t);
        t = ckt_terr(C, s, b + M1S_QGB, t);
    }
    return t;
}

/* the block's smallest step folded into the grid's (wide launch) */
__device__ void trunc_publish(const ngsf_ckt_t &C, double t)
{
    if (threadIdx.x == 0)
        atomicMin(&C.wide->tmin, (unsigned long long)__double_as_longlong(t));
}

/* CKTtrunc: DEVtrunc over all charges, min-reduced (a minimum is exact,
 * so the result does not depend on how the charges are shared out); in a
 * wide launch every block takes its share. */
__device__ double ckt_trunc(const ngsf_ckt_t &C, Ctl &s, double timeStep)
{
    double t;
    if (C.wide) {
        if (threadIdx.x == 0)
            wide_issue(C, s, NGSF_WIDE_TRUNC);
        t = block_min(s, trunc_share(C, s, threadIdx.x, gridDim.x * blockDim.x));
        trunc_publish(C, t);
        grid_sync(C, gridDim.x);
        __shared__ double tmin;
        if (threadIdx.x == 0)
            tmin = __longlong_as_double(
                (long long)*(volatile unsigned long long *)&C.wide->tmin);
        __syncthreads();
        t = tmin;
        __syncthreads();
    } else {
        t = block_min(s, trunc_share(C, s, threadIdx.x, blockDim.x));
    }
    return NG_MIN(2 * timeStep, t);
}

/* ---------------------------------------------------------------- */
/* breakpoints (analysis/cktsetbk.c, cktclrbk.c); thread 0 only        */
/* ---------------------------------------------------------------- */
__device__ int set_break(const ngsf_ckt_t &C, Ctl &s, double time)
{
    double *b = C.breaks;
    if (almost_equal_ulps(time, s.time, 3))
        return 0;
    if (s.time > time)
        return NGSF_E_BREAKS;
    for (int i = 0; i < s.nbreaks; i++) {
        if (b[i] > time) {
            if ((b[i] - time) <= C.opt.minbreak) {
                b[i] = time;
                return 0;
            }
            if (i > 0 && time - b[i - 1] <= C.opt.minbreak)
                return 0;
            if (s.nbreaks >= C.breakcap)
                return NGSF_E_BREAKS;
            for (int j = s.nbreaks; j > i; j--)
                b[j] = b[j - 1];
            b[i] = time;
            s.nbreaks++;
            return 0;
        }
    }
    if (time - b[s.nbreaks - 1] <= C.opt.minbreak)
        return 0;
    if (s.nbreaks >= C.breakcap)
        return NGSF_E_BREAKS;
    b[s.nbreaks++] = time;
    return 0;
}

__device__ void clr_break(const ngsf_ckt_t &C, Ctl &s)
{
    double *b = C.breaks;
    if (s.nbreaks > 2) {
        for (int j = 1; j < s.nbreaks; j++)
            b[j - 1] = b[j];
        s.nbreaks--;
    } else {
        b[0] = b[1];
        b[1] = C.opt.tstop;
    }
}

/* VSRCaccept / ISRCaccept breakpoint requests for PULSE and PWL
 * (vsrc/vsrcacct.c:23-330). */
__device__ int src_accept(const ngsf_ckt_t &C, Ctl &s, const ngsf_src_t &K)
{
    const ngsf_opts_t &o = C.opt;
    for (int i = 0; i < K.n; i++) {
        const double *cf = K.coef + (size_t)i * NGSF_MAX_COEFFS;
        int nc = K.ncoef[i];
        if (K.kind[i] == WF_PULSE) {
            double TD = nc > 2 ? cf[2] : 0.0;
            double TR = nc > 3 && cf[3] > 0.0 ? cf[3] : o.tstep;
            double TF = nc > 4 && cf[4] > 0.0 ? cf[4] : o.tstep;
            double PW = nc > 5 && cf[5] >= 0.0 ? cf[5] : 0.0;
            double PER = nc > 6 && cf[6] > 0.0 ? cf[6] : TR + TF + PW;
            double PHASE = nc > 7 ? cf[7] : 0.0;
            double time = s.time - TD;
            if (PHASE > 0.0) {
                double tmax = PHASE * PER;
                if (time > tmax)
                    continue;
            }
            if (s.time >= K.brk[i]) {
                double wait;
                if (time >= PER) {
                    double basetime = PER * floor(time / PER);
                    time -= basetime;
                }
                double atime = time + o.minbreak;
                if (atime < 0.0)
                    wait = -time;
                else if (atime < TR)
                    wait = TR - time;
                else if (atime < TR + PW)
                    wait = TR + PW - time;
                else if (atime < TR + PW + TF)
                    wait = TR + PW + TF - time;
                else
                    wait = PER - time;
                K.brk[i] = s.time + wait;
                int e = set_break(C, s, K.brk[i]);
                if (e)
                    return e;
                K.brk[i] -= o.minbreak;
            }
        } else if (K.kind[i] == WF_PWL) {
            if (s.time >= K.brk[i]) {
                double time = s.time;   /* no delay (td) support */
                double end = cf[nc - 2];
                if (time > end) {
                    K.brk[i] = o.tstop;
                    continue;
                }
                double atime = time + o.minbreak;
                for (int k = 0; k < nc; k += 2) {
                    if (cf[k] > atime) {
                        K.brk[i] = s.time + cf[k] - time;
                        int e = set_break(C, s, K.brk[i]);
                        if (e)
                            return e;
                        K.brk[i] -= o.minbreak;
                        break;
                    }
                }
            }
        }
    }
    return 0;
}

/* ---------------------------------------------------------------- */
/* NIiter                                                            */
/* ---------------------------------------------------------------- */
enum { PH_OP = 1, PH_NEXTTIME = 2, PH_STEP = 3, PH_STEP_NIITER = 4, PH_HELD = 5,
       PH_SYNC0 = 6, PH_SYNC1 = 7 };

__device__ void capture(const ngsf_ckt_t &C, Ctl &s, const Iter &it)
{
    int c = s.ncap;
    if (c >= C.capmax)
        return;
    for (int p = threadIdx.x; p < C.nnz; p += blockDim.x)
        C.cap_lux[(size_t)c * C.nnz + p] = C.ax[p];
    for (int r = threadIdx.x; r <= C.n; r += blockDim.x) {
        C.cap_rhs[(size_t)c * (C.n + 1) + r] = it.rhs[r];
        C.cap_rhs[(size_t)(C.capmax + c) * (C.n + 1) + r] = it.rhsOld[r];
    }
    if (threadIdx.x == 0) {
        C.cap_meta[4 * c + 0] = s.time;
        C.cap_meta[4 * c + 1] = s.delta;
        C.cap_meta[4 * c + 2] = s.mode;
        C.cap_meta[4 * c + 3] = s.order;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        s.ncap = c + 1;
    __syncthreads();
}

/* One NIiter call.  With resume set, the loaded matrix of the iteration
 * that asked for the re-pivot is already in ax / rhs and the host has just
 * planned new pivots for it: the iteration continues at the factorization.
 * Returns NGSF_NEED_REORDER when the host must choose pivots from the
 * current matrix first (the reference reorders at MODEINITJCT, at the
 * first MODEINITFIX iteration and at the first two iterations after
 * MODEINITTRAN: niiter.c:107-111, :328-346). */
__device__ int ni_iter(const ngsf_ckt_t &C, Ctl &s, int maxIter, bool resume)
{
    /* niiter.c raises the limit to 100; a start from the predictor's guess
     * keeps itl4, after which the step is retried from the plain start */
    if (maxIter < 100 && !(s.mode & NGSF_MODEGUESS))
        maxIter = 100;
    int iterno = resume ? s.savedIter : 0;
    for (;;) {
        Iter it = iter_ctx(C, s);
        int noncon;
        if (resume) {
            noncon = s.savedNoncon;
        } else {
            noncon = ckt_load(C, s, it);
            iterno++;
            if (C.wide && s.flag == NGSF_E_WATCHDOG) {
                /* a worker block stopped answering: end the run */
                if (threadIdx.x == 0)
                    s.numIter += iterno;
                __syncthreads();
                return NGSF_E_WATCHDOG;
            }
            if (C.capmax > 0)
                capture(C, s, it);
            bool want = (s.mode & NGSF_MODEINITJCT) ||
                        ((s.mode & NGSF_MODEINITTRAN) && iterno == 1) || s.shouldReorder;
            if (want) {
                __syncthreads();   /* every warp has read shouldReorder */
                if (threadIdx.x == 0) {
                    s.savedIter = iterno;
                    s.savedNoncon = noncon;
                    s.shouldReorder = 0;
                }
                __syncthreads();
                return NGSF_NEED_REORDER;
            }
        }
        long long tp = prof_t(C);
        int bad = lu_factor(C, s);
        prof_add(C, NGSF_P_FACTOR, tp);
        if (bad) {
            if (resume) {
                /* fresh pivots from this very matrix still fail: singular */
                if (threadIdx.x == 0) {
                    s.numIter += iterno;
                    s.badpivot++;
                }
                __syncthreads();
                return NGSF_E_SINGULAR;
            }
            if (threadIdx.x == 0) {
                s.savedIter = iterno;
                s.savedNoncon = noncon;
                s.badpivot++;
            }
            __syncthreads();
            return NGSF_NEED_REORDER;
        }
        resume = false;
        tp = prof_t(C);
        if (lu_solve(C, s, it.rhs)) {
            /* a solve wait ran out: stop with the step-budget status */
            if (threadIdx.x == 0)
                s.numIter += iterno;
            __syncthreads();
            return NGSF_E_WATCHDOG;
        }
        if (threadIdx.x == 0) {
            it.rhs[0] = 0;
            it.rhsOld[0] = 0;
        }
        __syncthreads();
        prof_add(C, NGSF_P_SOLVE, tp);
        if (C.prof && threadIdx.x == 0)
            C.prof[NGSF_P_ITERS]++;
        if (iterno > maxIter) {
            if (threadIdx.x == 0)
                s.numIter += iterno;
            __syncthreads();
            return NGSF_E_ITERLIM;
        }
        /* NIconvTest from the second iteration (niiter.c), or already after
         * the first when it started from the predictor's guess.  Then the
         * node voltages are tested against their guessed values; a branch
         * current does not enter the device loads (MNA is linear in it),
         * so the first solve's currents are the ones of the linearisation
         * at the guess and are taken as they are */
        const bool guess1 = (s.mode & NGSF_MODEGUESS) && iterno == 1;
        tp = prof_t(C);
        if (noncon == 0 && (iterno != 1 || guess1))
            noncon = conv_test(C, s, it, guess1);
        else
            noncon = 1;
        prof_add(C, NGSF_P_CONV, tp);
        int mode = s.mode & ~NGSF_MODEGUESS;
        int ret = -1, reorder = 0;
        if (mode & NGSF_MODEINITFLOAT) {
            if (noncon == 0)
                ret = NGSF_OK;
        } else if (mode & NGSF_MODEINITJCT) {
            mode = (mode & ~NGSF_INITF) | NGSF_MODEINITFIX;
            reorder = 1;
        } else if (mode & NGSF_MODEINITFIX) {
            if (noncon == 0)
                mode = (mode & ~NGSF_INITF) | NGSF_MODEINITFLOAT;
        } else if (mode & NGSF_MODEINITTRAN) {
            if (iterno <= 1)
                reorder = 1;
            mode = (mode & ~NGSF_INITF) | NGSF_MODEINITFLOAT;
        } else if (mode & NGSF_MODEINITPRED) {
            if (guess1 && noncon == 0)
                ret = NGSF_OK;
            mode = (mode & ~NGSF_INITF) | NGSF_MODEINITFLOAT;
        }
        if (guess1 && ret == NGSF_OK) {
            /* the accepted point keeps the guessed node voltages -- the
             * linearisation point the device states belong to, as the
             * reference reports its last linearisation point (NIiter returns
             * before its swap) -- with the branch currents of the solve */
            for (int i = 1 + threadIdx.x; i <= C.n; i += blockDim.x)
                if (!C.ntype[i])
                    it.rhsOld[i] = it.rhs[i];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (guess1 && ret == NGSF_OK)
                s.guessFirst++;
            s.mode &= ~NGSF_MODEGUESS;
            if (ret == NGSF_OK)
                s.numIter += iterno;
            else {
                s.mode = mode;
                if (reorder)
                    s.shouldReorder = 1;
                s.rhsSel ^= 1;   /* SWAP(rhs, rhsOld) */
            }
        }
        __syncthreads();
        if (ret == NGSF_OK)
            return NGSF_OK;
    }
}

/* NIcomCof (src/maths/ni/nicomcof.c:17-130).  Gear, orders 1 and 2 (the
 * engine keeps four state vectors): ag solves the corrector system whose
 * row j holds the j-th powers of (t_n - t_{n-i}) / delta, i = 0..order,
 * with right-hand side (0, -1/delta, 0, ..); the first column is
 * (1, 0, ..), so the elimination starts at row and column 1. */
__device__ void ni_comcof_gear(Ctl &s)
{
    const int q = s.order;
    double mat[3][3];
    for (int i = 0; i < 7; i++)
        s.ag[i] = 0;
    s.ag[1] = -1 / s.delta;
    double arg = 0;
    for (int i = 0; i <= q; i++)
        mat[0][i] = 1;
    for (int i = 1; i <= q; i++)
        mat[i][0] = 0;
    for (int i = 1; i <= q; i++) {
        arg += s.deltaOld[i - 1];
        double arg1 = 1;
        for (int j = 1; j <= q; j++) {
            arg1 *= arg / s.delta;
            mat[j][i] = arg1;
        }
    }
    for (int i = 1; i <= q; i++)
        for (int j = i + 1; j <= q; j++) {
            mat[j][i] /= mat[i][i];
            for (int k = i + 1; k <= q; k++)
                mat[j][k] -= mat[j][i] * mat[i][k];
        }
    for (int i = 1; i <= q; i++)
        for (int j = i + 1; j <= q; j++)
            s.ag[j] = s.ag[j] - mat[j][i] * s.ag[i];
    s.ag[q] /= mat[q][q];
    for (int i = q - 1; i >= 0; i--) {
        for (int j = i + 1; j <= q; j++)
            s.ag[i] = s.ag[i] - mat[i][j] * s.ag[j];
        s.ag[i] /= mat[i][i];
    }
}

__device__ void ni_comcof(const ngsf_ckt_t &C, Ctl &s)
{
    if (C.opt.method) {
        ni_comcof_gear(s);
        return;
    }
    if (s.order == 1) {
        s.ag[0] = 1 / s.delta;
        s.ag[1] = -1 / s.delta;
    } else {
        s.ag[0] = 1.0 / s.delta / (1.0 - C.opt.xmu);
        s.ag[1] = C.opt.xmu / (1.0 - C.opt.xmu);
    }
}

__device__ void copy_state(const ngsf_ckt_t &C, int dst, int src, const Ctl &s)
{
    double *d = C.states + (size_t)s.ring[dst] * C.nstates;
    const double *a = C.states + (size_t)s.ring[src] * C.nstates;
    for (int i = threadIdx.x; i < C.nstates; i += blockDim.x)
        d[i] = a[i];
    __syncthreads();
}

__device__ void dump_point(const ngsf_ckt_t &C, Ctl &s)
{
    int np = s.npoints;
    if (np < C.outcap) {
        Iter it = iter_ctx(C, s);
        double *row = C.out + (size_t)np * (1 + C.nprobe);
        for (int j = threadIdx.x; j < C.nprobe; j += blockDim.x)
            row[1 + j] = it.rhsOld[C.probe[j]];
        if (threadIdx.x == 0)
            row[0] = s.time;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        s.npoints = np + 1;
    __syncthreads();
}

/* ---------------------------------------------------------------- */
/* CKTop (src/spicelib/analysis/cktop.c:27-125) with its fallbacks    */
/* dynamic_gmin (:161-262), new_gmin (:329-422) and gillespie_src      */
/* (:436-654), as a resumable state machine                          */
/* ---------------------------------------------------------------- */
enum { OPP_NEWTON = 1, OPP_DG, OPP_DG_FINAL, OPP_NG, OPP_NG_FINAL, OPP_SS0, OPP_SSG, OPP_SS };

#define NGSF_GMINFACTOR 10.0
#define NGSF_ITL2 50

__device__ void op_zero(const ngsf_ckt_t &C, Ctl &s)
{
    Iter it = iter_ctx(C, s);
    for (int i = threadIdx.x; i <= C.n; i += blockDim.x)
        it.rhsOld[i] = 0;
    for (int i = threadIdx.x; i < C.nstates; i += blockDim.x)
        it.st0[i] = 0;
    __syncthreads();
}

__device__ void op_save(const ngsf_ckt_t &C, Ctl &s)
{
    Iter it = iter_ctx(C, s);
    for (int i = threadIdx.x; i <= C.n; i += blockDim.x)
        C.opsave_rhs[i] = it.rhsOld[i];
    for (int i = threadIdx.x; i < C.nstates; i += blockDim.x)
        C.opsave_st[i] = it.st0[i];
    __syncthreads();
}

__device__ void op_restore(const ngsf_ckt_t &C, Ctl &s)
{
    Iter it = iter_ctx(C, s);
    for (int i = threadIdx.x; i <= C.n; i += blockDim.x)
        it.rhsOld[i] = C.opsave_rhs[i];
    for (int i = threadIdx.x; i < C.nstates; i += blockDim.x)
        it.st0[i] = C.opsave_st[i];
    __syncthreads();
}

/* Returns 0 when the operating point converged, NGSF_NEED_REORDER when
 * paused, another code when every method failed. */
__device__ int op_run(const ngsf_ckt_t &C, Ctl &s, bool resume)
{
    const ngsf_opts_t &o = C.opt;
    const int firstmode = NGSF_MODETRANOP | NGSF_MODEINITJCT;
    const int contmode = NGSF_MODETRANOP | NGSF_MODEINITFLOAT;
    const double gshunt = 0.0;
    for (int guard = 0; guard < 100000; guard++) {
        const int ph = s.opPhase;
        if (ph == OPP_NEWTON) {
            int r = ni_iter(C, s, o.itl1, resume);
            resume = false;
            if (r == NGSF_NEED_REORDER || r == 0)
                return r;
            /* dynamic gmin stepping */
            op_zero(C, s);
            if (threadIdx.x == 0) {
                s.mode = firstmode;
                s.factor = NGSF_GMINFACTOR;
                s.oldGmin = 1e-2;
                s.diagGmin = s.oldGmin / s.factor;
                s.gtarget = NG_MAX(s.gmin, gshunt);
                s.itersBefore = s.numIter;
                s.opPhase = OPP_DG;
            }
            __syncthreads();
        } else if (ph == OPP_DG || ph == OPP_NG) {
            bool trueGmin = ph == OPP_NG;
            int r = ni_iter(C, s, NGSF_ITL2, resume);
            resume = false;
            if (r == NGSF_NEED_REORDER)
                return r;
            int iters = s.numIter - s.itersBefore;
            double g = trueGmin ? s.gmin : s.diagGmin;
            int action = 0;   /* 0 next step, 1 save, 2 restore, 3 done */
            if (r == 0) {
                action = g <= s.gtarget ? 3 : 1;
            } else {
                action = s.factor < 1.00005 ? 3 : 2;
            }
            if (action == 1)
                op_save(C, s);
            if (action == 2)
                op_restore(C, s);
            __syncthreads();   /* every warp has read gmin, factor, itersBefore */
            if (threadIdx.x == 0) {
                if (r == 0)
                    s.mode = contmode;
                if (action == 1) {
                    if (iters <= (NGSF_ITL2 / 4)) {
                        s.factor *= sqrt(s.factor);
                        if (s.factor > NGSF_GMINFACTOR)
                            s.factor = NGSF_GMINFACTOR;
                    }
                    if (iters > (3 * NGSF_ITL2 / 4))
                        s.factor = trueGmin ? NG_MAX(sqrt(s.factor), 3) : NG_MAX(sqrt(s.factor), 1.00005);
                    s.oldGmin = g;
                    if (g < s.factor * s.gtarget) {
                        s.factor = g / s.gtarget;
                        g = s.gtarget;
                    } else {
                        g /= s.factor;
                    }
                } else if (action == 2) {
                    s.factor = sqrt(sqrt(s.factor));
                    g = s.oldGmin / s.factor;
                }
                if (trueGmin)
                    s.gmin = g;
                else
                    s.diagGmin = g;
                if (action == 3) {
                    if (trueGmin) {
                        s.gmin = NG_MAX(s.startgmin, gshunt);
                        s.opPhase = OPP_NG_FINAL;
                    } else {
                        s.diagGmin = gshunt;
                        s.opPhase = OPP_DG_FINAL;
                    }
                }
                s.itersBefore = s.numIter;
            }
            __syncthreads();
        } else if (ph == OPP_DG_FINAL || ph == OPP_NG_FINAL) {
            int r = ni_iter(C, s, o.itl1, resume);
            resume = false;
            if (r == NGSF_NEED_REORDER || r == 0)
                return r;
            if (ph == OPP_DG_FINAL) {
                /* true gmin stepping */
                op_zero(C, s);
                if (threadIdx.x == 0) {
                    s.mode = firstmode;
                    s.startgmin = s.gmin;
                    s.factor = NGSF_GMINFACTOR;
                    s.oldGmin = 1e-2;
                    s.gmin = s.oldGmin / s.factor;
                    s.gtarget = NG_MAX(s.startgmin, gshunt);
                    s.itersBefore = s.numIter;
                    s.opPhase = OPP_NG;
                }
            } else {
                /* Gillespie source stepping */
                op_zero(C, s);
                if (threadIdx.x == 0) {
                    s.startgmin = s.gmin;   /* gminstart */
                    s.mode = firstmode;
                    s.srcFact = 0;
                    s.convFact = 0;
                    s.opPhase = OPP_SS0;
                }
            }
            __syncthreads();
        } else if (ph == OPP_SS0 || ph == OPP_SSG) {
            int r = ni_iter(C, s, NGSF_ITL2, resume);
            resume = false;
            if (r == NGSF_NEED_REORDER)
                return r;
            bool startRaise = false, failed = false;
            if (ph == OPP_SS0) {
                if (r != 0) {
                    if (threadIdx.x == 0) {
                        double dg = (gshunt <= 0) ? s.gmin : gshunt;
                        for (int i = 0; i < 10; i++)
                            dg *= 10;
                        s.diagGmin = dg;
                        s.gi = 0;
                        s.opPhase = OPP_SSG;
                    }
                    __syncthreads();
                } else {
                    startRaise = true;
                }
            } else {
                if (r != 0) {
                    failed = true;
                } else {
                    if (threadIdx.x == 0) {
                        s.diagGmin /= 10;
                        s.mode = contmode;
                        s.gi++;
                    }
                    __syncthreads();
                    if (s.gi > 10)
                        startRaise = true;
                }
                if (failed || startRaise) {
                    if (threadIdx.x == 0)
                        s.diagGmin = gshunt;
                    __syncthreads();
                }
            }
            if (failed) {
                if (threadIdx.x == 0)
                    s.srcFact = 1;
                __syncthreads();
                return NGSF_E_ITERLIM;
            }
            if (startRaise) {
                op_save(C, s);
                if (threadIdx.x == 0) {
                    s.raise = 0.001;
                    s.srcFact = s.convFact + s.raise;
                    s.itersBefore = s.numIter;
                    s.opPhase = OPP_SS;
                }
                __syncthreads();
            }
        } else if (ph == OPP_SS) {
            int r = ni_iter(C, s, NGSF_ITL2, resume);
            resume = false;
            if (r == NGSF_NEED_REORDER)
                return r;
            int iters = s.numIter - s.itersBefore;
            bool brk = false;
            if (r == 0) {
                op_save(C, s);
            } else {
                brk = s.srcFact - s.convFact < 1e-8;
                if (!brk) {
                    /* restore uses the rhsOld selected below: swap first */
                    op_restore(C, s);
                }
            }
            __syncthreads();   /* every warp has read srcFact and convFact */
            if (threadIdx.x == 0) {
                s.mode = contmode;
                if (r == 0) {
                    s.convFact = s.srcFact;
                    s.srcFact = s.convFact + s.raise;
                    if (iters <= (NGSF_ITL2 / 4))
                        s.raise *= 1.5;
                    if (iters > (3 * NGSF_ITL2 / 4))
                        s.raise *= 0.5;
                } else if (!brk) {
                    s.raise /= 10;
                    if (s.raise > 0.01)
                        s.raise = 0.01;
                    s.srcFact = s.convFact;
                }
                if (s.srcFact > 1)
                    s.srcFact = 1;
                s.itersBefore = s.numIter;
            }
            __syncthreads();
            if (brk || !((s.raise >= 1e-7) && (s.convFact < 1))) {
                int ok = s.convFact == 1;
                if (threadIdx.x == 0) {
                    s.diagGmin = s.gmin = s.startgmin;
                    s.srcFact = 1;
                }
                __syncthreads();
                return ok ? 0 : NGSF_E_ITERLIM;
            }
        } else {
            return NGSF_E_NOOP;
        }
    }
    return NGSF_E_NOOP;
}

/* ---------------------------------------------------------------- */
/* DCtran, as a resumable state machine                              */
/* ---------------------------------------------------------------- */
/* With hold set, a circuit stops (NGSF_HELD) once its first transient step
 * is accepted -- after the operating point and the re-pivots that the
 * reference asks for at MODEINITJCT, MODEINITFIX and MODEINITTRAN -- and a
 * held circuit stays held; the host releases the batch once no circuit
 * still waits for new pivots, so those early pauses cost short launches
 * instead of one long launch each. */
/* A synchronised run stops at sharedsync, loc 1 (dctran.c:937-960), after
 * the step's verdict: redostep 0 (accepted; the phase is already nextTime)
 * or 1 (rejected; the time is already moved back and delta cut).  The host
 * hands time, delta and olddelta to the caller and resumes in PH_SYNC1. */
__device__ int sync_stop(Ctl &s, int redostep)
{
    __syncthreads();   /* every warp has read the phase and the step state */
    if (threadIdx.x == 0) {
        s.phase = PH_SYNC1;
        s.syncLoc = 2;
        s.syncRedo = redostep;
        s.syncReply = 0;
    }
    __syncthreads();
    return NGSF_HELD;
}

__device__ int dc_tran(const ngsf_ckt_t &C, Ctl &s, long long maxSteps, bool resume, bool hold)
{
    const ngsf_opts_t &o = C.opt;
    const int maxOrder = o.maxord;
    if (!resume) {
        if (threadIdx.x == 0) {
            s.delta = NG_MIN(o.tstop / 100, o.tstep) / 10;   /* local 'delta' */
            s.delta0 = s.delta;
            C.breaks[0] = 0;
            C.breaks[1] = o.tstop;
            s.nbreaks = 2;
            s.time = 0;
            s.firsttime = 1;
            s.mode = NGSF_MODETRANOP | NGSF_MODEINITJCT;
            s.order = 1;
            s.phase = PH_OP;
            s.opPhase = OPP_NEWTON;
            s.steps = 0;
        }
        __syncthreads();
    }
    if (s.phase == PH_OP) {
        /* CKTop: Newton on the operating point, then its fallbacks */
        int conv = op_run(C, s, resume);
        resume = false;
        if (conv == NGSF_NEED_REORDER)
            return conv;
        if (conv != 0)
            return conv == NGSF_E_SINGULAR ? conv : NGSF_E_NOOP;
        if (threadIdx.x == 0) {
            s.opiter = s.numIter;
            s.timePts++;
            s.order = 1;
            for (int i = 0; i < 7; i++)
                s.deltaOld[i] = o.tmax;
            s.delta = s.delta0;              /* CKTdelta = delta */
            s.saveDelta = o.tstop / 50;
            s.mode = NGSF_MODETRAN | NGSF_MODEINITTRAN;
            s.ag[0] = s.ag[1] = 0;
            s.phase = PH_NEXTTIME;
        }
        __syncthreads();
        copy_state(C, 1, 0, s);
    }

    for (;;) {
        if (s.phase == PH_HELD) {
            if (hold || s.time >= C.pause_at)
                return NGSF_HELD;
            resume = false;
        } else if (s.phase == PH_NEXTTIME) {
            /* nextTime: CKTaccept, clear passed breakpoint, dump, finish test */
            if (threadIdx.x == 0) {
                int e = src_accept(C, s, C.vsrc);
                if (!e)
                    e = src_accept(C, s, C.isrc);
                s.flag = e;
                if (!e && s.time > C.breaks[0])
                    clr_break(C, s);
                s.accepted++;
            }
            __syncthreads();
            if (s.flag)
                return s.flag;
            if (s.time >= o.tstart)
                dump_point(C, s);
            pred_accept(C, s);
            if (almost_equal_ulps(s.time, o.tstop, 100))
                return NGSF_OK;
            if (s.steps + 1 > maxSteps)
                return NGSF_E_WATCHDOG;
            if (s.time >= C.pause_at) {
                /* end of a window: stop here; the next window resumes */
                __syncthreads();   /* every warp has read time */
                if (threadIdx.x == 0)
                    s.phase = PH_HELD;
                __syncthreads();
                return NGSF_HELD;
            }
            if (hold && s.accepted == 2) {
                __syncthreads();   /* every warp has read accepted */
                if (threadIdx.x == 0)
                    s.phase = PH_HELD;
                __syncthreads();
                return NGSF_HELD;
            }
        }
        if (s.phase == PH_NEXTTIME || s.phase == PH_HELD) {
            /* resume: */
            __syncthreads();   /* every warp has read time, steps and the phase */
            if (threadIdx.x == 0) {
                s.steps++;
                double *b = C.breaks;
                s.delta = NG_MIN(s.delta, o.tmax);
                if (almost_equal_ulps(s.time, b[0], 100) || b[0] - s.time <= o.delmin) {
                    s.order = 1;
                    s.delta = NG_MIN(s.delta, .1 * NG_MIN(s.saveDelta, b[1] - b[0]));
                    if (s.firsttime)
                        s.delta /= 10;
                }
                while ((b[0] <= s.time + o.minbreak || almost_equal_ulps(b[0], s.time, 100)) &&
                       b[0] < o.tstop)
                    clr_break(C, s);
                if (s.time + s.delta > b[0]) {
                    s.saveDelta = s.delta;
                    s.delta = b[0] - s.time;
                } else if (s.time + 1.9 * s.delta > b[0]) {
                    s.saveDelta = s.delta;
                    s.delta = (b[0] - s.time) / 2.;
                }
                s.phase = PH_SYNC0;
                s.syncLoc = C.sync ? 1 : 0;
                s.syncRedo = 0;
            }
            __syncthreads();
            /* sharedsync, loc 0 (dctran.c:598-601): a synchronised run
             * stops here; the caller may change delta */
            if (C.sync)
                return NGSF_HELD;
        }
        if (s.phase == PH_SYNC0) {
            resume = false;
            __syncthreads();   /* every warp has read the phase */
            if (threadIdx.x == 0) {
                /* a caller's 1 here only counts a rejection (the time moves
                 * back by an olddelta of 0; dctran ignores the value) */
                if (s.syncLoc && s.syncReply)
                    s.rejected++;
                s.syncLoc = s.syncReply = 0;
                for (int i = 5; i >= 0; i--)
                    s.deltaOld[i + 1] = s.deltaOld[i];
                s.deltaOld[0] = s.delta;
                int temp = s.ring[maxOrder + 1];
                for (int i = maxOrder; i >= 0; i--)
                    s.ring[i + 1] = s.ring[i];
                s.ring[0] = temp;
                s.phase = PH_STEP;
            }
            __syncthreads();
        }
        if (s.phase == PH_SYNC1) {
            /* the caller's answer at sharedsync loc 1: an accepted step
             * goes on to nextTime unless the caller asks to redo it (the
             * time then moves back by olddelta and the step counts as
             * rejected, sharedspice.c sharedsync); a rejected step is
             * tried again with the delta in force */
            resume = false;
            __syncthreads();   /* every warp has read the phase */
            if (threadIdx.x == 0) {
                const bool redo = s.syncRedo || s.syncReply;
                if (!s.syncRedo && s.syncReply) {
                    s.time -= s.olddelta;
                    s.rejected++;
                }
                s.syncLoc = s.syncReply = s.syncRedo = 0;
                if (redo) {
                    s.steps++;
                    s.phase = PH_STEP;
                } else {
                    s.phase = PH_NEXTTIME;
                }
            }
            __syncthreads();
            if (s.phase == PH_STEP && s.steps > maxSteps)
                return NGSF_E_WATCHDOG;
            continue;
        }
        if (s.phase == PH_STEP) {
            __syncthreads();   /* every warp has read the phase */
            if (threadIdx.x == 0) {
                s.olddelta = s.delta;
                s.time += s.delta;
                s.deltaOld[0] = s.delta;
                ni_comcof(C, s);
                s.iters0 = s.numIter;
                s.phase = PH_STEP_NIITER;
                s.guessUsed = 0;
            }
            __syncthreads();
            if (C.pred.kind && s.histCount >= 3 && (s.mode & NGSF_MODEINITPRED) && !s.guessOff)
                pred_guess(C, s);
        }
        /* PH_STEP_NIITER */
        int converged = ni_iter(C, s, o.itl4, resume);
        resume = false;
        if (converged == NGSF_NEED_REORDER)
            return converged;
        if (s.guessUsed && converged != 0 && converged != NGSF_E_SINGULAR &&
            converged != NGSF_E_WATCHDOG) {
            /* Newton from the predictor's guess missed itl4: the same step
             * again from the plain start (INITPRED) */
            __syncthreads();   /* every warp has read guessUsed */
            if (threadIdx.x == 0) {
                s.tranIter += s.numIter - s.iters0;
                s.time -= s.delta;
                s.guessOff = 1;
                s.guessUsed = 0;
                s.guessFalls++;
                s.mode = NGSF_MODETRAN | NGSF_MODEINITPRED;
                s.phase = PH_STEP;
            }
            __syncthreads();
            continue;
        }
        if (threadIdx.x == 0) {
            s.tranIter += s.numIter - s.iters0;
            s.timePts++;
            s.mode = NGSF_MODETRAN | NGSF_MODEINITPRED;
        }
        __syncthreads();
        if (s.firsttime) {
            copy_state(C, 2, 1, s);
            copy_state(C, 3, 1, s);
        }
        if (converged == NGSF_E_SINGULAR)
            return converged;
        if (converged != 0) {
            if (threadIdx.x == 0) {
                s.time = s.time - s.delta;
                s.rejected++;
                s.delta = s.delta / 8;
                if (s.firsttime)
                    s.mode = NGSF_MODETRAN | NGSF_MODEINITTRAN;
                s.order = 1;
                /* the retry factors with pivots chosen on its own matrix
                 * (the reference re-pivots the retry of the first step
                 * through MODEINITTRAN; here every retry after a Newton
                 * failure does: a failing Newton is the symptom of pivots
                 * gone stale, and fresh ones cost one host pause) */
                if (C.retry_repivot)
                    s.shouldReorder = 1;
            }
            __syncthreads();
        } else {
            if (s.firsttime) {
                __syncthreads();
                if (threadIdx.x == 0) {
                    s.firsttime = 0;
                    s.phase = PH_NEXTTIME;
                }
                __syncthreads();
                if (C.sync)
                    return sync_stop(s, 0);
                continue;
            }
            const long long tt = prof_t(C);
            double newdelta = ckt_trunc(C, s, s.delta);
            prof_add(C, NGSF_P_TRUNC, tt);
            if (newdelta > .9 * s.delta) {
                if (s.order == 1 && maxOrder > 1) {
                    __syncthreads();   /* every warp has read the order */
                    if (threadIdx.x == 0)
                        s.order = 2;
                    __syncthreads();
                    newdelta = ckt_trunc(C, s, s.delta);
                    if (threadIdx.x == 0 && newdelta <= 1.05 * s.delta)
                        s.order = 1;
                    __syncthreads();
                }
                if (threadIdx.x == 0) {
                    s.delta = newdelta;
                    s.phase = PH_NEXTTIME;
                }
                __syncthreads();
                if (C.sync)
                    return sync_stop(s, 0);
                continue;
            } else {
                __syncthreads();   /* every warp has compared against delta */
                if (threadIdx.x == 0) {
                    s.time = s.time - s.delta;
                    s.rejected++;
                    s.delta = newdelta;
                }
                __syncthreads();
            }
        }
        if (s.delta <= o.delmin) {
            if (s.olddelta > o.delmin) {
                if (threadIdx.x == 0)
                    s.delta = o.delmin;
                __syncthreads();
            } else {
                return NGSF_E_TIMESTEP;
            }
        }
        if (C.sync)
            return sync_stop(s, 1);
        if (threadIdx.x == 0) {
            s.steps++;
            s.phase = PH_STEP;
        }
        __syncthreads();
        if (s.steps > maxSteps)
            return NGSF_E_WATCHDOG;
    }
}

/* launch modes */
#define RUN_FRESH 0
#define RUN_RESUME 1
#define RUN_PROBE 2
#define RUN_HOLD 4     /* or-ed into RUN_FRESH / RUN_RESUME: stop after the first step */

__device__ void run_circuit(const ngsf_ckt_t &C, Ctl &s, int runMode, long long maxSteps);

/* Batched launch: block b runs the transient of circuit order[b] (the
 * host orders the circuits largest first).  The hardware block scheduler
 * starts a waiting block on an SM as soon as a block there retires, so
 * circuits of uneven size keep every SM busy and the largest ones start
 * first (longest-processing-time order). */
/* Registers per thread of the transient kernels: an explicit cap of 255
 * (the BSIM4 evaluation keeps everything in registers, no spills).  With
 * only __launch_bounds__(256) the compiler settles on 128 registers and
 * spills about 1.2 KB a thread.  NGSF_TRAN_MAXNREG (a build-time define)
 * sets another cap for experiments. */
#ifndef NGSF_TRAN_MAXNREG
#define NGSF_TRAN_MAXNREG 255
#endif
#define NGSF_TRAN_BOUNDS __maxnreg__(NGSF_TRAN_MAXNREG)
#if NGSF_IN(1)
__global__ void NGSF_TRAN_BOUNDS
tran_kernel(const ngsf_ckt_t *ckts, const int *order, int nckt, int runMode,
            long long maxSteps, int solveCap, int gnnBytes)
{
    extern __shared__ __align__(16) unsigned char ngsf_dyn[];
    __shared__ Ctl s;
    __shared__ __align__(16) ngsf_ckt_t Cs;
    const int q = blockIdx.x;
    if (q >= nckt)
        return;
    pred_block_init(gnnBytes >= PRED_STAGE_BYTES ? ngsf_dyn + solveCap : nullptr);
    {
        const unsigned long long *src = (const unsigned long long *)(ckts + order[q]);
        unsigned long long *dst = (unsigned long long *)&Cs;
        for (int w = threadIdx.x; w < (int)(sizeof(ngsf_ckt_t) / 8); w += blockDim.x)
            dst[w] = src[w];
    }
    __syncthreads();
    if (threadIdx.x == 0)
        Cs.wide = nullptr;
    __syncthreads();
    solve_buffers_init(Cs, ngsf_dyn, solveCap);
    run_circuit(Cs, s, runMode, maxSteps);
    pred_block_fini();
}

#endif  /* NGSF_IN(1) */
#if NGSF_IN(2)
/* One circuit over the whole (cooperative) grid: block 0 runs the
 * transient, the other blocks evaluate transistors on its command. */
__global__ void NGSF_TRAN_BOUNDS
tran_wide_kernel(const ngsf_ckt_t *ckt, int runMode, long long maxSteps, int solveCap,
                 int gnnBytes)
{
    extern __shared__ __align__(16) unsigned char ngsf_dyn[];
    __shared__ Ctl s;
    __shared__ __align__(16) ngsf_ckt_t Cs;
    if (threadIdx.x == 0)
        g_barGen = g_fbarGen = 0;
    {
        const unsigned long long *src = (const unsigned long long *)ckt;
        unsigned long long *dst = (unsigned long long *)&Cs;
        for (int w = threadIdx.x; w < (int)(sizeof(ngsf_ckt_t) / 8); w += blockDim.x)
            dst[w] = src[w];
    }
    __syncthreads();
    if (blockIdx.x != 0) {
        wide_worker(Cs, s);
        return;
    }
    solve_buffers_init(Cs, ngsf_dyn, solveCap);
    pred_block_init(gnnBytes >= PRED_STAGE_BYTES ? ngsf_dyn + solveCap : nullptr);
    run_circuit(Cs, s, runMode, maxSteps);
    pred_block_fini();
    if (threadIdx.x == 0)
        wide_issue(Cs, s, NGSF_WIDE_EXIT);
}

#endif  /* NGSF_IN(2) */
__device__ void run_circuit(const ngsf_ckt_t &C, Ctl &s, int runMode, long long maxSteps)
{
    const bool hold = (runMode & RUN_HOLD) != 0;
    runMode &= ~RUN_HOLD;
    if (runMode == RUN_FRESH && C.run_resume)
        runMode = RUN_RESUME;   /* the next window of a paused run */
    if (C.prof && threadIdx.x == 0 && runMode == RUN_FRESH)
        for (int k = 0; k < NGSF_P_COUNT; k++)
            C.prof[k] = 0;
    __syncthreads();
    const long long tRun = prof_t(C);
    if (runMode == RUN_RESUME) {
        const int *src = (const int *)C.ctlsave;
        int *dst = (int *)&s;
        for (int w = threadIdx.x; w < (int)(sizeof(Ctl) / 4); w += blockDim.x)
            dst[w] = src[w];
        __syncthreads();
    } else {
        if (threadIdx.x == 0) {
            for (int i = 0; i < 4; i++)
                s.ring[i] = i;
            s.rhsSel = 0;
            s.status = 0;
            s.accepted = s.rejected = s.numIter = s.tranIter = s.timePts = 0;
            s.npoints = s.ncap = s.badpivot = s.opiter = 0;
            s.order = 1;
            s.delta = 0;
            s.time = 0;
            s.flag = 0;
            s.phase = 0;
            s.shouldReorder = 0;
            s.savedIter = s.savedNoncon = s.iters0 = s.reorders = 0;
            s.steps = 0;
            s.tcur = s.th0 = s.th1 = 0.0;
            s.histCount = s.guessOff = s.guessUsed = 0;
            s.guessSteps = s.guessFirst = s.guessFalls = 0;
            s.gmin = C.opt.gmin;
            s.diagGmin = 0.0;
            s.srcFact = 1.0;
            s.opPhase = 0;
            s.syncLoc = s.syncRedo = s.syncReply = 0;
            for (int i = 0; i < 7; i++) {
                s.ag[i] = 0;
                s.deltaOld[i] = 0;
            }
        }
        __syncthreads();
        /* zero per-run buffers: states, rhs, per-instance memories */
        for (size_t i = threadIdx.x; i < (size_t)4 * C.nstates; i += blockDim.x)
            C.states[i] = 0.0;
        for (int i = threadIdx.x; i <= C.n; i += blockDim.x) {
            C.rhs[i] = 0.0;
            C.rhsOld[i] = 0.0;
        }
        for (size_t i = threadIdx.x; i < (size_t)M1H_COUNT * C.mos1.n; i += blockDim.x)
            C.mos1.h[i] = 0.0;
        for (size_t i = threadIdx.x; i < (size_t)B4H_COUNT * C.bsim4.n; i += blockDim.x)
            C.bsim4.h[i] = 0.0;
        for (int i = threadIdx.x; i < C.vsrc.n; i += blockDim.x)
            C.vsrc.brk[i] = -1.0;
        for (int i = threadIdx.x; i < C.isrc.n; i += blockDim.x)
            C.isrc.brk[i] = -1.0;
        __syncthreads();
    }
    int status;
    if (runMode == RUN_PROBE) {
        if (threadIdx.x == 0)
            s.mode = NGSF_MODETRANOP | NGSF_MODEINITJCT;
        __syncthreads();
        Iter it = iter_ctx(C, s);
        ckt_load(C, s, it);
        status = NGSF_OK;
    } else {
        status = dc_tran(C, s, maxSteps, runMode == RUN_RESUME, hold);
    }
    __syncthreads();
    if (status == NGSF_NEED_REORDER || status == NGSF_HELD) {
        if (threadIdx.x == 0 && status == NGSF_NEED_REORDER)
            s.reorders++;
        __syncthreads();
        int *dst = (int *)C.ctlsave;
        const int *src = (const int *)&s;
        for (int w = threadIdx.x; w < (int)(sizeof(Ctl) / 4); w += blockDim.x)
            dst[w] = src[w];
    }
    if (threadIdx.x == 0) {
        C.result[NGSF_R_STATUS] = status;
        C.result[NGSF_R_NPOINTS] = s.npoints;
        C.result[NGSF_R_ACCEPTED] = s.accepted;
        C.result[NGSF_R_REJECTED] = s.rejected;
        C.result[NGSF_R_NUMITER] = s.numIter;
        C.result[NGSF_R_TRANITER] = s.tranIter;
        C.result[NGSF_R_TIMEPTS] = s.timePts;
        C.result[NGSF_R_NCAP] = s.ncap;
        C.result[NGSF_R_OPITER] = s.opiter;
        C.result[NGSF_R_BADPIVOT] = s.badpivot;
        C.result[NGSF_R_REORDERS] = s.reorders;
        C.result[NGSF_R_GUESSES] = s.guessSteps;
        C.result[NGSF_R_GUESS1] = s.guessFirst;
        C.result[NGSF_R_FALLBACKS] = s.guessFalls;
        C.fresult[NGSF_F_TIME] = s.time;
        C.fresult[NGSF_F_DELTA] = s.delta;
        C.fresult[NGSF_F_DIAGGMIN] = s.diagGmin;
        C.result[NGSF_R_SYNCLOC] = status == NGSF_HELD ? s.syncLoc : 0;
        C.result[NGSF_R_SYNCREDO] = s.syncRedo;
        C.fresult[NGSF_F_OLDDELTA] = s.olddelta;
    }
    prof_add(C, NGSF_P_TOTAL, tRun);
}

}  // namespace

#if NGSF_IN(3)
/* ---------------------------------------------------------------- */
/* First-iteration stamps without allocation                          */
/* ---------------------------------------------------------------- */
/* The operating-point initialisation load of one circuit (CKTload in
 * MODETRANOP | MODEINITJCT from zero state: the matrix and right-hand side
 * that the first Newton iteration hands to the factorization), with every
 * mutable array of the launch -- state vectors, right-hand sides, stamp
 * slots, matrix values, per-instance memories, result words -- placed in
 * this file-scope device array instead of device memory owned by the
 * circuit.  8 MiB: a few thousand transistors; larger circuits are refused. */
#define NGSF_STATIC_SCRATCH_BYTES (8u << 20)
static __device__ __align__(256) unsigned char g_static_scratch[NGSF_STATIC_SCRATCH_BYTES];

__global__ void __launch_bounds__(NGSF_THREADS) stamp_static_kernel(ngsf_ckt_t C)
{
    __shared__ Ctl s;
    __shared__ __align__(16) ngsf_ckt_t Cs;
    if (threadIdx.x == 0)
        Cs = C;
    __syncthreads();
    if (threadIdx.x == 0) {      /* RUN_PROBE stamps only: no solve buffers */
        g_sw = nullptr;
        g_sflag = nullptr;
        g_psm = nullptr;
    }
    run_circuit(Cs, s, RUN_PROBE, 0);
}

/* ---------------------------------------------------------------- */
/* Operator surface: one device operation on a circuit's arrays,      */
/* outside the transient -- CKTload / DEVload of chosen device types, */
/* SMPluFac, SMPsolve, NIconvTest, CKTtrunc -- on one block, with the */
/* control scalars the caller gives (ngsf_ckt_load and friends)        */
/* ---------------------------------------------------------------- */
struct OpArgs {
    int op, mode, order, types;
    double time, delta, deltaOld[3], ag0, ag1, ag2, gmin, srcFact, diagGmin;
};
enum { OPK_LOAD = 1, OPK_LUFAC, OPK_SOLVE, OPK_CONV, OPK_TRUNC };

/* first stamp slot of each device type in table order (bsim4, cap, dio,
 * isrc, mos1, res, vsrc), then the slot count: the compiler lays the
 * types' slot blocks out in this order */
__device__ void type_slot_starts(const ngsf_ckt_t &C, int st[8])
{
    st[0] = C.bsim4.stamp0;
    st[1] = C.cap.stamp0;
    st[2] = C.dio.stamp0;
    st[3] = C.isrc.stamp0;
    st[4] = C.mos1.stamp0;
    st[5] = C.res.stamp0;
    st[6] = C.vsrc.stamp0;
    st[7] = C.nstamp;
}

/* CKTload restricted to the device types in `types` (bit k = type k of
 * the table order): the other types' stamp slots are cleared, so the
 * gather sums exactly the selected DEVload contributions, in the
 * reference's order.  All types: the whole CKTload. */
__device__ int op_load(const ngsf_ckt_t &C, Ctl &s, const Iter &it, int types)
{
    const int t = threadIdx.x, T = blockDim.x;
    int st[8];
    type_slot_starts(C, st);
    int nc = 0;
    if (types & (1 << NGSF_DEV_BSIM4))
        for (int i = t; i < C.bsim4.n; i += T)
            nc |= bsim4_load_one(C, s, it, i);
    if (types & (1 << NGSF_DEV_CAP))
        cap_load(C, s, it, t, T);
    if (types & (1 << NGSF_DEV_DIO))
        for (int i = t; i < C.dio.n; i += T)
            nc |= dio_load_one(C, s, it, i);
    if (types & (1 << NGSF_DEV_MOS1))
        for (int i = t; i < C.mos1.n; i += T)
            nc |= mos1_load_one(C, s, it, i);
    if (types & (1 << NGSF_DEV_RES))
        res_load(C, t, T);
    if (types & ((1 << NGSF_DEV_VSRC) | (1 << NGSF_DEV_ISRC)))
        src_load(C, s);
    __syncthreads();
    for (int k = 0; k < NGSF_DEV_TYPES; k++)
        if (!(types & (1 << k)))
            for (int q = st[k] + t; q < st[k + 1]; q += T)
                C.stampv[q] = 0.0;
    nc = block_or(s, nc);   /* includes __syncthreads: stamps visible */
    gather(C, it, t, T, t >> 5, (int)(blockDim.x >> 5));
    __syncthreads();
    gather_heavy_combine(C, it);
    __syncthreads();
    return nc;
}

__global__ void __launch_bounds__(NGSF_THREADS)
op_kernel(const ngsf_ckt_t *ckt, OpArgs a, int solveCap, int *iout, double *dout)
{
    extern __shared__ __align__(16) unsigned char ngsf_dyn[];
    __shared__ Ctl s;
    __shared__ __align__(16) ngsf_ckt_t Cs;
    {
        const unsigned long long *src = (const unsigned long long *)ckt;
        unsigned long long *dst = (unsigned long long *)&Cs;
        for (int w = threadIdx.x; w < (int)(sizeof(ngsf_ckt_t) / 8); w += blockDim.x)
            dst[w] = src[w];
        unsigned long long *z = (unsigned long long *)&s;
        for (int w = threadIdx.x; w < (int)(sizeof(Ctl) / 8); w += blockDim.x)
            z[w] = 0ull;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Cs.wide = nullptr;
        g_psm = nullptr;
        s.time = a.time;
        s.delta = a.delta;
        for (int k = 0; k < 3; k++)
            s.deltaOld[k] = a.deltaOld[k];
        s.ag[0] = a.ag0;
        s.ag[1] = a.ag1;
        s.ag[2] = a.ag2;
        s.order = a.order;
        s.mode = a.mode;
        s.gmin = a.gmin;
        s.srcFact = a.srcFact;
        s.diagGmin = a.diagGmin;
        for (int k = 0; k < 4; k++)
            s.ring[k] = k;
        s.rhsSel = 0;
    }
    __syncthreads();
    solve_buffers_init(Cs, ngsf_dyn, solveCap);
    Iter it = iter_ctx(Cs, s);
    int r = 0;
    double d = 0.0;
    switch (a.op) {
    case OPK_LOAD:
        r = op_load(Cs, s, it, a.types);
        break;
    case OPK_LUFAC:
        r = lu_factor(Cs, s);
        break;
    case OPK_SOLVE:
        r = lu_solve(Cs, s, it.rhs);
        break;
    case OPK_CONV:
        r = conv_test(Cs, s, it);
        break;
    case OPK_TRUNC:
        d = ckt_trunc(Cs, s, a.delta);
        break;
    default:
        r = -1;
    }
    if (threadIdx.x == 0) {
        iout[0] = r;
        dout[0] = d;
    }
}

/* Stand-alone device evaluation over the whole grid: every thread of the
 * grid evaluates the devices of the selected types one instance at a time
 * (the same device functions the transient calls), `reps` times, with no
 * gather.  It times the FP64-bound half of CKTload on its own. */
__global__ void __launch_bounds__(NGSF_THREADS)
eval_kernel(const ngsf_ckt_t *ckt, OpArgs a, int reps)
{
    __shared__ Ctl s;
    __shared__ __align__(16) ngsf_ckt_t Cs;
    {
        const unsigned long long *src = (const unsigned long long *)ckt;
        unsigned long long *dst = (unsigned long long *)&Cs;
        for (int w = threadIdx.x; w < (int)(sizeof(ngsf_ckt_t) / 8); w += blockDim.x)
            dst[w] = src[w];
        unsigned long long *z = (unsigned long long *)&s;
        for (int w = threadIdx.x; w < (int)(sizeof(Ctl) / 8); w += blockDim.x)
            z[w] = 0ull;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s.time = a.time;
        s.delta = a.delta;
        for (int k = 0; k < 3; k++)
            s.deltaOld[k] = a.deltaOld[k];
        s.ag[0] = a.ag0;
        s.ag[1] = a.ag1;
        s.ag[2] = a.ag2;
        s.order = a.order;
        s.mode = a.mode;
        s.gmin = a.gmin;
        s.srcFact = a.srcFact;
        for (int k = 0; k < 4; k++)
            s.ring[k] = k;
    }
    __syncthreads();
    const Iter it = iter_ctx(Cs, s);
    const int t = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
    for (int r = 0; r < reps; r++) {
        if (a.types & (1 << NGSF_DEV_BSIM4))
            for (int i = t; i < Cs.bsim4.n; i += T)
                bsim4_load_one(Cs, s, it, i);
        if (a.types & (1 << NGSF_DEV_MOS1))
            for (int i = t; i < Cs.mos1.n; i += T)
                mos1_load_one(Cs, s, it, i);
        if (a.types & (1 << NGSF_DEV_DIO))
            for (int i = t; i < Cs.dio.n; i += T)
                dio_load_one(Cs, s, it, i);
    }
}

/* FP64 throughput probe: independent fused multiply-add chains per
 * thread (2 flops each), the result kept live through one store. */
__global__ void fp64_peak_kernel(double *out, int iters)
{
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-10, a2 = a0 + 2e-10, a3 = a0 + 3e-10;
    double a4 = a0 + 4e-10, a5 = a0 + 5e-10, a6 = a0 + 6e-10, a7 = a0 + 7e-10;
    const double m = 0.999999999, c = 1e-12;
    for (int i = 0; i < iters; i++) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
        a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    const double r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678)
        out[blockIdx.x] = r;
}

#endif  /* NGSF_IN(3) */
static_assert(sizeof(Ctl) <= NGSF_WIDE_CTL_BYTES, "control block does not fit the wide hand-over");

#if NGSF_IN(1)
extern "C" int ngsf_ctl_bytes(void) { return (int)sizeof(Ctl); }

/* The caller's answer to a sharedsync stop, written into the paused run's
 * saved control block: the delta of the next step and the return value
 * (1: redo the step). */
extern "C" cudaError_t ngsf_sync_write(void *ctlsave, double delta, int reply)
{
    cudaError_t e = cudaMemcpy((char *)ctlsave + offsetof(Ctl, delta), &delta, sizeof(double),
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy((char *)ctlsave + offsetof(Ctl, syncReply), &reply, sizeof(int),
                       cudaMemcpyHostToDevice);
    return e;
}

#endif  /* NGSF_IN(1) */
#if NGSF_IN(2)
namespace {
cudaError_t allow_dyn_smem(const void *fn);
}

/* Blocks a cooperative wide launch can keep resident on this device. */
extern "C" int ngsf_wide_blocks(void)
{
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    /* the launch may ask for the largest dynamic allocation: allow it first */
    if (allow_dyn_smem((const void *)tran_wide_kernel) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tran_wide_kernel, NGSF_THREADS,
                                                      NGSF_SOLVE_SMEM_MAX + PRED_STAGE_BYTES) !=
        cudaSuccess)
        return 0;
    return sms * per;
}

#endif  /* NGSF_IN(2) */
extern "C" const ngsf_ckt_t *ngsf_internal_desc(const ngsf_handle *h);
extern "C" void ngsf_internal_set_error(const char *msg);

#if NGSF_IN(3)
namespace {

/* Device address of g_static_scratch on the current device, looked up on
 * every call (cudaGetSymbolAddress allocates nothing and is cheap): a
 * cached address would go stale when the module is reloaded after a
 * cudaDeviceReset. */
void *static_scratch(std::string &err)
{
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) {
        err = std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e);
        return nullptr;
    }
    return p;
}

}  // namespace

extern "C" NGSF_API int ngsf_stamp_initial_static(const ngsf_handle *h, double *ax, double *rhs)
{
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d) {
        ngsf_internal_set_error("ngsf_stamp_initial_static: null or host-only handle");
        return -1;
    }
    /* layout of the mutable arrays, each on a 256-byte boundary */
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    const size_t n1 = (size_t)d->n + 1;
    size_t o_states = take(4 * ((size_t)d->nstates + 1) * sizeof(double));
    size_t o_rhs = take(n1 * sizeof(double));
    size_t o_rhsOld = take(n1 * sizeof(double));
    size_t o_stampv = take((size_t)d->nstamp * sizeof(double));
    size_t o_ax = take((size_t)d->nnz * sizeof(double));
    size_t o_m1h = take((size_t)M1H_COUNT * d->mos1.n * sizeof(double));
    size_t o_b4h = take((size_t)B4H_COUNT * d->bsim4.n * sizeof(double));
    size_t o_vbrk = take((size_t)d->vsrc.n * sizeof(double));
    size_t o_ibrk = take((size_t)d->isrc.n * sizeof(double));
    size_t o_res = take(NGSF_R_ALL * sizeof(int));
    size_t o_fres = take(NGSF_F_ALL * sizeof(double));
    size_t o_hpart = take((size_t)d->nhchunk * sizeof(double));
    if (off > NGSF_STATIC_SCRATCH_BYTES) {
        std::string m = "ngsf_stamp_initial_static: the circuit needs " + std::to_string(off) +
                        " bytes of scratch, more than the static " +
                        std::to_string((size_t)NGSF_STATIC_SCRATCH_BYTES) + " bytes";
        ngsf_internal_set_error(m.c_str());
        return -1;
    }
    std::string err;
    unsigned char *base = (unsigned char *)static_scratch(err);
    if (!base) {
        ngsf_internal_set_error(err.c_str());
        return -1;
    }
    ngsf_ckt_t c = *d;
    c.states = (double *)(base + o_states);
    c.rhs = (double *)(base + o_rhs);
    c.rhsOld = (double *)(base + o_rhsOld);
    c.stampv = (double *)(base + o_stampv);
    c.ax = (double *)(base + o_ax);
    c.mos1.h = (double *)(base + o_m1h);
    c.bsim4.h = (double *)(base + o_b4h);
    c.vsrc.brk = (double *)(base + o_vbrk);
    c.isrc.brk = (double *)(base + o_ibrk);
    c.result = (int *)(base + o_res);
    c.hpart = (double *)(base + o_hpart);
    c.fresult = (double *)(base + o_fres);
    c.capmax = 0;
    c.wide = nullptr;
    c.pred.kind = 0;
    c.prof = nullptr;
    c.pause_at = INFINITY;
    c.run_resume = 0;
    stamp_static_kernel<<<1, NGSF_THREADS>>>(c);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && ax)
        e = cudaMemcpy(ax, c.ax, (size_t)d->nnz * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && rhs)
        e = cudaMemcpy(rhs, c.rhs, n1 * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        ngsf_internal_set_error(cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

/* Dynamic shared memory for the solve workspace of circuits with n
 * unknowns: (n+1) doubles rounded to 128 bytes, or 0 when that exceeds
 * NGSF_SOLVE_SMEM_MAX (the solve then works in global memory). */
#endif  /* NGSF_IN(3) */
#if NGSF_IN(1)
extern "C" int ngsf_solve_smem_bytes(int n, int tags)
{
    /* the solve vector, then (dependency-driven solves only) the row tags;
     * no more than that, since the reservation shrinks the L1 cache */
    size_t v = ((size_t)(n + 1) * sizeof(double) + 127) & ~(size_t)127;
    size_t b = (v + (size_t)n * sizeof(int) + 127) & ~(size_t)127;
    if (tags && b <= (size_t)NGSF_SOLVE_SMEM_MAX)
        return (int)b;
    return v <= (size_t)NGSF_SOLVE_SMEM_MAX ? (int)v : 0;
}

/* staging of the predictor's network tiles (0 when no circuit has one) */
extern "C" int ngsf_pred_smem_bytes(int any) { return any ? PRED_STAGE_BYTES : 0; }

#endif  /* NGSF_IN(1) */
#if NGSF_IN(2) || NGSF_IN(3)
namespace {
cudaError_t allow_dyn_smem(const void *fn)
{
    static std::mutex mu;
    static const void *doneFn[16] = {nullptr};
    static int doneDev[16];
    static int ndone = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < ndone; i++)
        if (doneFn[i] == fn && doneDev[i] == dev)
            return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             NGSF_SOLVE_SMEM_MAX + PRED_STAGE_BYTES);
    if (e == cudaSuccess && ndone < 16) {
        doneFn[ndone] = fn;
        doneDev[ndone++] = dev;
    }
    return e;
}
}  // namespace

#endif  /* NGSF_IN(2) || NGSF_IN(3) */
#if NGSF_IN(2)
extern "C" cudaError_t ngsf_launch_tran_wide(const ngsf_ckt_t *d_ckt, int nblocks, int runMode,
                                             long long maxSteps, int solveCap, int gnnBytes,
                                             cudaStream_t stream)
{
    cudaError_t e = allow_dyn_smem((const void *)tran_wide_kernel);
    if (e != cudaSuccess)
        return e;
    void *args[] = {(void *)&d_ckt, (void *)&runMode, (void *)&maxSteps, (void *)&solveCap,
                    (void *)&gnnBytes};
    return cudaLaunchCooperativeKernel((const void *)tran_wide_kernel, dim3(nblocks),
                                       dim3(NGSF_THREADS), args,
                                       (size_t)solveCap + (size_t)gnnBytes, stream);
}

#endif  /* NGSF_IN(2) */
#if NGSF_IN(1)
/* circuit blocks of the batched launch one SM holds at once; *regs and
 * *smem (may be NULL) receive the kernel's registers per thread and static
 * shared bytes */
extern "C" int ngsf_tran_occupancy(int threads, int dynSmem, int *regs, int *smem)
{
    int per = 0;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, (const void *)tran_kernel) == cudaSuccess) {
        if (regs)
            *regs = fa.numRegs;
        if (smem)
            *smem = (int)fa.sharedSizeBytes;
    }
    if (cudaFuncSetAttribute((const void *)tran_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, dynSmem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tran_kernel, threads, dynSmem) !=
            cudaSuccess)
        return 0;
    return per;
}

/* threads: 64, 128 or 256 per circuit block.  Every loop of the kernel is
 * strided by the block size and every sum keeps its order, so the result
 * does not depend on it; fewer threads let several circuits share an SM
 * (255 registers a thread: two 128-thread blocks, or four 64-thread
 * blocks). */
extern "C" cudaError_t ngsf_launch_tran(const ngsf_ckt_t *d_ckts, const int *d_order, int nckt,
                                        int runMode, long long maxSteps, int solveCap,
                                        int gnnBytes, int threads, cudaStream_t stream)
{
    if (nckt <= 0)
        return cudaSuccess;
    if (threads != 64 && threads != 128)
        threads = NGSF_THREADS;
    /* the dynamic shared memory this launch uses, no more: a larger
     * reservation takes its room from the L1 cache, which the
     * refactorization's and solves' loads hit (factor values staged in
     * 209 KB of shared memory per block instead ran 6 % slower) */
    cudaError_t e = cudaFuncSetAttribute((const void *)tran_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         solveCap + gnnBytes);
    if (e != cudaSuccess)
        return e;
    tran_kernel<<<nckt, threads, (size_t)solveCap + (size_t)gnnBytes, stream>>>(
        d_ckts, d_order, nckt, runMode, maxSteps, solveCap, gnnBytes);
    return cudaGetLastError();
}

#endif  /* NGSF_IN(1) */
#if NGSF_IN(3)
/* ---------------------------------------------------------------- */
/* Operator surface, host side (declared in ngspice_gb300.h)          */
/* ---------------------------------------------------------------- */
extern "C" const ngsf_ckt_t *ngsf_internal_ddesc(const ngsf_handle *h);

namespace {

OpArgs op_args(int op, const ngsf_point *pt, int types)
{
    OpArgs a{};
    a.op = op;
    a.types = types;
    if (pt) {
        a.mode = pt->mode;
        a.order = pt->order;
        a.time = pt->time;
        a.delta = pt->delta;
        for (int k = 0; k < 3; k++)
            a.deltaOld[k] = pt->deltaOld[k];
        a.ag0 = pt->ag[0];
        a.ag1 = pt->ag[1];
        a.ag2 = pt->ag[2];
        a.gmin = pt->gmin;
        a.srcFact = pt->srcFact;
        a.diagGmin = pt->diagGmin;
    }
    return a;
}

/* one op_kernel launch on circuit h; *r / *dv receive its result words */
int launch_op(const ngsf_handle *h, const OpArgs &a, int *r, double *dv, const char *who)
{
    const ngsf_ckt_t *hd = ngsf_internal_desc(h), *dd = ngsf_internal_ddesc(h);
    if (!hd || !dd) {
        ngsf_internal_set_error((std::string(who) + ": null or host-only handle").c_str());
        return -1;
    }
    int *d_i = nullptr;
    cudaError_t e = cudaMalloc(&d_i, 16);
    if (e == cudaSuccess)
        e = allow_dyn_smem((const void *)op_kernel);
    const int solveCap = ngsf_solve_smem_bytes(hd->n, hd->solve_sf);
    if (e == cudaSuccess) {
        op_kernel<<<1, NGSF_THREADS, (size_t)solveCap>>>(dd, a, solveCap, d_i,
                                                          (double *)(d_i + 2));
        e = cudaGetLastError();
    }
    int ri[4] = {0};
    if (e == cudaSuccess)
        e = cudaMemcpy(ri, d_i, 16, cudaMemcpyDeviceToHost);
    if (d_i)
        cudaFree(d_i);
    if (e != cudaSuccess) {
        ngsf_internal_set_error((std::string(who) + ": " + cudaGetErrorString(e)).c_str());
        return -1;
    }
    if (r)
        *r = ri[0];
    if (dv)
        memcpy(dv, ri + 2, sizeof(double));
    return 0;
}

int put(void *dst, const void *src, size_t bytes, const char *who)
{
    if (!src || !bytes)
        return 0;
    cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        ngsf_internal_set_error((std::string(who) + ": " + cudaGetErrorString(e)).c_str());
        return -1;
    }
    return 0;
}

int get(void *dst, const void *src, size_t bytes, const char *who)
{
    if (!dst || !bytes)
        return 0;
    cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        ngsf_internal_set_error((std::string(who) + ": " + cudaGetErrorString(e)).c_str());
        return -1;
    }
    return 0;
}

/* the linearisation point: rhsOld, CKTstates[0..nvec-1], BSIM4von */
int put_point(const ngsf_ckt_t *d, const double *rhsOld, const double *states, int nvec,
              const double *von, const char *who)
{
    if (nvec < 0 || nvec > 4) {
        ngsf_internal_set_error((std::string(who) + ": nvec must be 0..4").c_str());
        return -1;
    }
    const size_t n1 = (size_t)d->n + 1;
    if (put(d->rhsOld, rhsOld, n1 * sizeof(double), who))
        return -1;
    if (states && put(d->states, states, (size_t)nvec * d->nstates * sizeof(double), who))
        return -1;
    if (von && d->bsim4.n > 0 &&
        put(d->bsim4.h + (size_t)B4H_VON * d->bsim4.n, von, (size_t)d->bsim4.n * sizeof(double),
            who))
        return -1;
    return 0;
}

}  // namespace

extern "C" NGSF_API int ngsf_ckt_load(ngsf_handle *h, const ngsf_point *pt, int types,
                                      const double *rhsOld, const double *states, int nvec,
                                      const double *von, double *ax, double *rhs, int *noncon)
{
    const char *who = "ngsf_ckt_load";
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || !pt) {
        ngsf_internal_set_error("ngsf_ckt_load: null handle or point");
        return -1;
    }
    const int starts[8] = {d->bsim4.stamp0, d->cap.stamp0, d->dio.stamp0, d->isrc.stamp0,
                           d->mos1.stamp0,  d->res.stamp0, d->vsrc.stamp0, d->nstamp};
    for (int k = 0; k < NGSF_DEV_TYPES; k++)
        if (starts[k] > starts[k + 1]) {
            ngsf_internal_set_error("ngsf_ckt_load: stamp slot blocks out of table order");
            return -1;
        }
    if (put_point(d, rhsOld, states, nvec, von, who))
        return -1;
    int nc = 0;
    if (launch_op(h, op_args(OPK_LOAD, pt, types & ((1 << NGSF_DEV_TYPES) - 1)), &nc, nullptr,
                  who))
        return -1;
    if (get(ax, d->ax, (size_t)d->nnz * sizeof(double), who) ||
        get(rhs, d->rhs, ((size_t)d->n + 1) * sizeof(double), who))
        return -1;
    if (noncon)
        *noncon = nc;
    return 0;
}

extern "C" NGSF_API int ngsf_ckt_read_states(const ngsf_handle *h, double *states, int nvec)
{
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || nvec < 0 || nvec > 4) {
        ngsf_internal_set_error("ngsf_ckt_read_states: null handle or nvec outside 0..4");
        return -1;
    }
    return get(states, d->states, (size_t)nvec * d->nstates * sizeof(double),
               "ngsf_ckt_read_states");
}

extern "C" NGSF_API int ngsf_ckt_trunc(ngsf_handle *h, const ngsf_point *pt,
                                       const double *states, int nvec, double *timestep)
{
    const char *who = "ngsf_ckt_trunc";
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || !pt || pt->order < 1 || pt->order > 2) {
        ngsf_internal_set_error("ngsf_ckt_trunc: null handle or point, or order outside 1..2");
        return -1;
    }
    if (put_point(d, nullptr, states, nvec, nullptr, who))
        return -1;
    double t = 0;
    if (launch_op(h, op_args(OPK_TRUNC, pt, 0), nullptr, &t, who))
        return -1;
    if (timestep)
        *timestep = t;
    return 0;
}

extern "C" NGSF_API int ngsf_ni_convtest(ngsf_handle *h, const double *rhs, const double *rhsOld,
                                         int *noncon)
{
    const char *who = "ngsf_ni_convtest";
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || !rhs || !rhsOld) {
        ngsf_internal_set_error("ngsf_ni_convtest: null handle or vector");
        return -1;
    }
    const size_t b = ((size_t)d->n + 1) * sizeof(double);
    if (put(d->rhs, rhs, b, who) || put(d->rhsOld, rhsOld, b, who))
        return -1;
    int nc = 0;
    if (launch_op(h, op_args(OPK_CONV, nullptr, 0), &nc, nullptr, who))
        return -1;
    if (noncon)
        *noncon = nc;
    return 0;
}

extern "C" NGSF_API int ngsf_smp_set_matrix(ngsf_handle *h, const double *ax)
{
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || !ax) {
        ngsf_internal_set_error("ngsf_smp_set_matrix: null handle or values");
        return -1;
    }
    return put(d->ax, ax, (size_t)d->nnz * sizeof(double), "ngsf_smp_set_matrix");
}

extern "C" NGSF_API int ngsf_smp_get_matrix(const ngsf_handle *h, double *ax)
{
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || !ax) {
        ngsf_internal_set_error("ngsf_smp_get_matrix: null handle or buffer");
        return -1;
    }
    return get(ax, d->ax, (size_t)d->nnz * sizeof(double), "ngsf_smp_get_matrix");
}

extern "C" NGSF_API int ngsf_smp_lufac(ngsf_handle *h, double diag_gmin)
{
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d) {
        ngsf_internal_set_error("ngsf_smp_lufac: null handle");
        return -1;
    }
    if (d->nlu <= 0) {
        ngsf_internal_set_error("ngsf_smp_lufac: no pivot sequence yet (call ngsf_smp_reorder)");
        return -1;
    }
    ngsf_point pt{};
    pt.diagGmin = diag_gmin;
    int bad = 0;
    if (launch_op(h, op_args(OPK_LUFAC, &pt, 0), &bad, nullptr, "ngsf_smp_lufac"))
        return -1;
    return bad ? NGSF_E_SINGULAR : 0;
}

extern "C" NGSF_API int ngsf_smp_solve(ngsf_handle *h, double *rhs)
{
    const char *who = "ngsf_smp_solve";
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || !rhs || d->nlu <= 0) {
        ngsf_internal_set_error("ngsf_smp_solve: null handle or vector, or no factor yet");
        return -1;
    }
    const size_t b = ((size_t)d->n + 1) * sizeof(double);
    if (put(d->rhs, rhs, b, who))
        return -1;
    int late = 0;
    if (launch_op(h, op_args(OPK_SOLVE, nullptr, 0), &late, nullptr, who))
        return -1;
    if (late) {
        ngsf_internal_set_error("ngsf_smp_solve: a bounded wait of the solve ran out");
        return -1;
    }
    if (get(rhs, d->rhs, b, who))
        return -1;
    rhs[0] = 0.0;
    return 0;
}

/* the engine side of ngsf_smp_reorder (api.cpp plans the pivots) */
extern "C" int ngsf_internal_lufac(ngsf_handle *h, double diag_gmin)
{
    return ngsf_smp_lufac(h, diag_gmin);
}

extern "C" NGSF_API int ngsf_eval_bench(ngsf_handle *h, const ngsf_point *pt, int types,
                                        int reps, int blocks, double *seconds)
{
    const char *who = "ngsf_eval_bench";
    const ngsf_ckt_t *dd = ngsf_internal_ddesc(h);
    if (!dd || !pt || reps < 1) {
        ngsf_internal_set_error("ngsf_eval_bench: null handle or point, or reps < 1");
        return -1;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (blocks <= 0)
        blocks = sms;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    OpArgs a = op_args(0, pt, types);
    if (e == cudaSuccess) {
        eval_kernel<<<blocks, NGSF_THREADS>>>(dd, a, 1);   /* warm-up */
        cudaEventRecord(e0, 0);
        eval_kernel<<<blocks, NGSF_THREADS>>>(dd, a, reps);
        cudaEventRecord(e1, 0);
        e = cudaEventSynchronize(e1);
    }
    if (e == cudaSuccess)
        e = cudaGetLastError();
    float ms = 0;
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        ngsf_internal_set_error((std::string(who) + ": " + cudaGetErrorString(e)).c_str());
        return -1;
    }
    if (seconds)
        *seconds = ms * 1e-3;
    return 0;
}

extern "C" NGSF_API int ngsf_fp64_peak(double *flops_per_second)
{
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *d = nullptr;
    const int blocks = 8 * (sms > 0 ? sms : 1), threads = 256, iters = 1 << 14;
    if (e == cudaSuccess)
        e = cudaMalloc(&d, (size_t)blocks * sizeof(double));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    float best = 0;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(e0, 0);
        fp64_peak_kernel<<<blocks, threads>>>(d, iters);
        cudaEventRecord(e1, 0);
        e = cudaEventSynchronize(e1);
        float ms = 0;
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0 || ms < best))
            best = ms;
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (d)
        cudaFree(d);
    if (e != cudaSuccess || best <= 0) {
        ngsf_internal_set_error(e != cudaSuccess ? cudaGetErrorString(e) : "fp64 probe: no time");
        return -1;
    }
    if (flops_per_second)
        *flops_per_second = 2.0 * 8.0 * (double)iters * blocks * threads / (best * 1e-3);
    return 0;
}
#endif  /* NGSF_IN(3) */
