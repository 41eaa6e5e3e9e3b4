/*
 * Device-resident data layout of one compiled circuit, shared by the host
 * compiler (C++) and the CUDA transient engine.
 *
 * Everything below is structure-of-arrays: field f of instance i of a device
 * type lives at  base[f * n + i],  so the threads of a warp, which take
 * consecutive instances, read and write consecutive addresses.
 *
 * Equation numbering follows the reference: equation 0 is ground, 1..n are
 * the unknowns, in the order CKTnames reports them.  Matrix stamps never
 * address ground; a stamp whose row or column is ground is dropped at
 * compile time (the reference writes it to a trash cell,
 * src/maths/KLU/klusmp.c:418-440).
 */
#ifndef NGSF_TYPES_H
#define NGSF_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CKTmode bits, same values as src/include/ngspice/cktdefs.h:171-199 */
#define NGSF_MODETRAN        0x1
#define NGSF_MODEDC          0x70
#define NGSF_MODEDCOP        0x10
#define NGSF_MODETRANOP      0x20
#define NGSF_MODEDCTRANCURVE 0x40
#define NGSF_INITF           0x3f00
#define NGSF_MODEINITFLOAT   0x100
#define NGSF_MODEINITJCT     0x200
#define NGSF_MODEINITFIX     0x400
#define NGSF_MODEINITSMSIG   0x800
#define NGSF_MODEINITTRAN    0x1000
#define NGSF_MODEINITPRED    0x2000
#define NGSF_MODEUIC         0x10000
/* engine-only bit (no reference counterpart): the first Newton iteration of
 * a timestep starts from the predictor's guess in rhsOld (INITPRED state
 * copies, terminal voltages from rhsOld) */
#define NGSF_MODEGUESS       0x100000

/* error codes, same values as src/include/ngspice/sperror.h */
#define NGSF_OK         0
#define NGSF_E_ITERLIM  101   /* E_ITERLIM  = E_PRIVATE + 1 */
#define NGSF_E_TIMESTEP 106   /* E_TIMESTEP */
#define NGSF_E_SINGULAR 102   /* E_SINGULAR */
#define NGSF_E_ORDER    103
#define NGSF_E_NOOP     110   /* operating point not found */
#define NGSF_E_BREAKS   120   /* breakpoint table overflow */
#define NGSF_E_WATCHDOG 121   /* step budget exhausted */
#define NGSF_NEED_REORDER (-2) /* paused: host must choose new pivots */
#define NGSF_HELD (-3)        /* paused after the first transient step while
                                 other circuits of the batch re-pivot */

/* -------- MOS1 (level 1) --------------------------------------------- */
enum {
    M1N_D, M1N_G, M1N_S, M1N_B, M1N_DP, M1N_SP, M1N_COUNT
};
/* constant per-instance parameters, computed once on the host exactly as
 * MOS1temp (mos1temp.c) and the head of MOS1load (mos1load.c:131-154) do */
enum {
    M1P_TYPE, M1P_VT, M1P_DSAT, M1P_SSAT, M1P_CGSO, M1P_CGDO, M1P_CGBO,
    M1P_BETA, M1P_COX, M1P_TPHI, M1P_TVBI, M1P_TVTO, M1P_GAMMA, M1P_LAMBDA,
    M1P_SVCRIT, M1P_DVCRIT, M1P_CBS, M1P_CBSSW, M1P_CBD, M1P_CBDSW,
    M1P_TDEPCAP, M1P_TBULKPOT, M1P_F2S, M1P_F3S, M1P_F4S, M1P_F2D, M1P_F3D,
    M1P_F4D, M1P_MJ, M1P_MJSW, M1P_GDRAIN, M1P_GSOURCE, M1P_OFF,
    M1P_ICVDS, M1P_ICVGS, M1P_ICVBS, M1P_COUNT
};
/* per-instance values the reference keeps in the instance struct between
 * Newton iterations (MOS1mode, MOS1von, MOS1cd, ...) */
enum {
    M1H_MODE, M1H_VON, M1H_VDSAT, M1H_CD, M1H_CBS, M1H_CBD, M1H_GBS,
    M1H_GBD, M1H_GM, M1H_GDS, M1H_GMBS, M1H_CAPBS, M1H_CAPBD, M1H_COUNT
};
/* state vector layout (mos1defs.h: MOS1vbd .. MOS1cqbs, 17 doubles) */
enum {
    M1S_VBD, M1S_VBS, M1S_VGS, M1S_VDS, M1S_CAPGS, M1S_QGS, M1S_CQGS,
    M1S_CAPGD, M1S_QGD, M1S_CQGD, M1S_CAPGB, M1S_QGB, M1S_CQGB, M1S_QBD,
    M1S_CQBD, M1S_QBS, M1S_CQBS, M1S_COUNT
};
#define M1_NSTAMP_MAT 22
#define M1_NSTAMP_RHS 4
#define M1_NSTAMP (M1_NSTAMP_MAT + M1_NSTAMP_RHS)

typedef struct {
    int n;
    const int *node;      /* [M1N_COUNT][n] */
    const int *st;        /* [n] state offset */
    const double *p;      /* [M1P_COUNT][n] */
    double *h;            /* [M1H_COUNT][n] */
    int stamp0;           /* first stamp slot; slot = stamp0 + k*n + i */
} ngsf_mos1_t;

/* -------- BSIM4 (field enums in bsim4.h) ------------------------------- */
typedef struct {
    int n;
    const int *node;      /* [B4N_COUNT][n] */
    const int *st;        /* [n] state offset */
    const double *p;      /* [B4P_COUNT][n] */
    double *h;            /* [B4H_COUNT][n] */
    int stamp0;           /* first stamp slot; slot = stamp0 + k*n + i */
} ngsf_bsim4_t;

/* -------- diode (field enums in dio.h) --------------------------------- */
typedef struct {
    int n;
    const int *node;      /* [DIN_COUNT][n] */
    const int *st;
    const double *p;      /* [DIP_COUNT][n] */
    double *h;            /* unused */
    int stamp0;
} ngsf_dio_t;

/* -------- resistor / capacitor --------------------------------------- */
typedef struct {
    int n;
    const int *node;      /* [2][n] */
    const double *g;      /* [n] conductance (RESconduct) */
    int stamp0;           /* 4 matrix stamps per instance */
} ngsf_res_t;

typedef struct {
    int n;
    const int *node;      /* [2][n] */
    const int *st;        /* [n] state offset (qcap, ccap) */
    const double *c;      /* [n] capacitance (CAPcapac) */
    const double *m;      /* [n] multiplier (CAPm) */
    const double *ic;     /* [n] initial condition (CAPinitCond) */
    int stamp0;           /* 4 matrix + 2 rhs stamps per instance */
} ngsf_cap_t;

/* -------- independent sources ----------------------------------------- */
enum { WF_DC = 0, WF_PULSE = 1, WF_SINE = 2, WF_EXP = 3, WF_PWL = 4 };
#define NGSF_MAX_COEFFS 64

typedef struct {
    int n;
    const int *node;      /* [3][n]: pos, neg, branch (branch unused by isrc) */
    const int *kind;      /* [n] waveform kind */
    const int *ncoef;     /* [n] VSRCfunctionOrder */
    const double *coef;   /* [n][NGSF_MAX_COEFFS] (AoS: per-instance tables) */
    const double *dc;     /* [n] dc value */
    const int *dcgiven;   /* [n] */
    const double *m;      /* [n] multiplier (isrc only) */
    double *brk;          /* [n] next breakpoint request (VSRCbreak_time) */
    int stamp0;           /* vsrc: 4 matrix + 1 rhs; isrc: 2 rhs */
} ngsf_src_t;

/* -------- whole circuit ----------------------------------------------- */
typedef struct {
    double reltol, abstol, vntol, chgtol, trtol, gmin, pivtol, pivrel, xmu;
    double tstep, tstop, tstart, tmax, delmin, minbreak, temp;
    int itl1, itl4, maxord, method, uic, order_init;
} ngsf_opts_t;

/* -------- wide launch: one circuit over a cooperative grid ------------ *
 * Block 0 runs the transient; the other blocks wait for its commands and
 * evaluate their share of the device instances.  The words are handed over
 * with device-scope release/acquire; every wait is bounded. */
#define NGSF_WIDE_CTL_BYTES 1024
#define NGSF_HCHUNK 1024
enum { NGSF_WIDE_LOAD = 1, NGSF_WIDE_EXIT = 2, NGSF_WIDE_FACTOR = 3, NGSF_WIDE_TRUNC = 4 };
typedef struct {
    int seq;              /* command number, bumped by block 0 (release) */
    int cmd;              /* NGSF_WIDE_* */
    int done;             /* blocks that finished the current command */
    int noncon;           /* OR of the workers' convergence flags */
    int err;              /* 1: a bounded wait ran out */
    int bad;              /* OR of the blocks' pivot checks (factor command) */
    unsigned long long bar;  /* grid barrier: arrivals since the launch */
    unsigned long long gen;  /* grid barrier: generations completed (last arriver) */
    unsigned long long fbar, fgen;  /* the same for the refactorization's block group */
    unsigned long long tmin;        /* CKTtrunc: bits of the smallest step (positive doubles
                                     * order like their bit patterns) */
    unsigned long long ctl[NGSF_WIDE_CTL_BYTES / 8];  /* block 0's control words */
} ngsf_wide_t;

/* -------- learned Newton predictor (engine addition) ------------------ *
 * Per circuit: the voltage unknowns, their neighbour graph and terminal
 * counts, the last three accepted solutions, activations, and BF16 copies
 * of the network (kind 2).  kind 0: off; 1: linear extrapolation guess;
 * 2: linear extrapolation plus the network's correction. */
#define NGSF_PRED_VSCALE 0.05
#define NGSF_PRED_VOUT 0.005    /* V: unit of the network's correction */
#define NGSF_PRED_RATIO_MAX 4.0
#define NGSF_PRED_QUIET 1e-4     /* V: activity at which the correction is halved */
typedef struct {
    int kind;
    int nv;                       /* voltage unknowns */
    const int *vnode;             /* [nv] equation index 1..n */
    const int *gptr, *gidx;       /* neighbour CSR over 0..nv-1 */
    const float *dinv;            /* [nv] 1 / degree */
    const float *stat;            /* [nv][6] log(1 + terminal counts) */
    float *Ha, *Hb;               /* [nv rounded to 128][64] activations */
    double *cur, *h0, *h1;        /* [n+1] v_n, v_n-1, v_n-2 */
    const unsigned short *WinT;   /* bf16 [64][16] */
    const unsigned short *WT[3];  /* bf16 [64][128] */
    const unsigned short *WoutT;  /* bf16 [16][64] */
    const float *bin, *bl[3], *bout;
} ngsf_pred_t;

typedef struct {
    /* sizes */
    int n;                /* unknowns (equations 1..n) */
    int nstates;          /* doubles per state vector */
    int nstamp;           /* stamp slots */
    int nlu;              /* nonzeros of L+U (including the diagonal) */
    int nlevels;          /* column levels of the numeric factorization */
    int nslevels;         /* row levels of the triangular solves */

    ngsf_opts_t opt;

    /* devices, in the reference device-table order for load/trunc/conv */
    ngsf_bsim4_t bsim4;
    ngsf_dio_t dio;
    ngsf_mos1_t mos1;
    ngsf_res_t res;
    ngsf_cap_t cap;
    ngsf_src_t vsrc;
    ngsf_src_t isrc;

    const int *ntype;     /* [n+1] 1 = voltage node, 0 = current (branch) */

    /* stamping: ax[p] = sum of stampv[gsrc[gptr[p]..gptr[p+1])] for each
     * matrix entry p (CSC order); rhs[i] = sum of stampv[rsrc[rptr[i]..]]
     * for equations i = 1..n.  Lists are in the reference load order, so
     * every cell is summed in the same order CKTload adds into it. */
    int nnz;
    double *stampv;       /* [nstamp] */
    double *ax;           /* [nnz] */
    const int *gptr, *gsrc;
    int nheavy;           /* entries summed by a warp (more than 64 terms) */
    const int *heavy;     /* matrix entry p >= 0, or rhs row r as -r-1 */
    const int *rptr, *rsrc;
    const int *a_lupos;   /* [nnz] position of each entry in lux */
    const int *a_diag;    /* [n] entry index of A(j,j), -1 when absent */

    /* LU (left-looking, static pivots, structurally symmetric fill) */
    double *lux;          /* [nlu] */
    const int *lvl_ptr;   /* [nlevels+1] into lvl_col */
    const int *lvl_col;   /* columns (pivot order) grouped by level */
    const int *cdiag;     /* [n] lux position of U(j,j) */
    const int *cend;      /* [n] one past the last L(:,j) position */
    const int *cbeg;      /* [n] first position of column j */
    const int *kptr;      /* [n+1] into kdep/kpos/kseg: U entries of column j */
    const int *kdep;      /* column k of each U(k,j) (ascending) */
    const int *kpos;      /* lux position of U(k,j) */
    const int *kseg;      /* [.. +1] into upd: updates from column k to j */
    const int *upd_dst;   /* lux position in column j */
    const int *upd_src;   /* lux position of L(i,k) */
    const int *prow;      /* [n] original equation (1-based) of pivot row k */
    const int *pcol;      /* [n] original equation (1-based) of pivot col k */
    /* triangular solves, row oriented over pivot indices */
    const int *fl_ptr, *fl_row;   /* forward levels: rows grouped by level */
    const int *bl_ptr, *bl_row;   /* backward levels */
    int nflevels, nblevels;
    const int *lr_ptr, *lr_col, *lr_pos;  /* L rows: (k, lux pos) for m<k */
    /* the solve's view, refreshed after each refactorization: per row in
     * level order {row, first term, end, 0} (fdesc forward, bdesc backward)
     * and the L/U values in term order (lval[q] = lux[lr_pos[q]]) */
    const int *fdesc, *bdesc;
    double *lval, *uval;
    int nlterm, nuterm;
    const int *ur_ptr, *ur_col, *ur_pos;  /* U rows: (m, lux pos) for m>k */
    const int *fh_ptr, *fh_row;   /* per forward level: rows reduced by a warp */
    const int *bh_ptr, *bh_row;   /* per backward level: rows reduced by a warp */
    /* right-looking schedule (used when rl_levels > 0): per level, its
     * pivot columns, the L entries to divide by their pivot, and the
     * destinations with their lists of (L pos, U pos) products */
    int rl_levels;
    /* refactorization shape in a wide launch, 0 = built-in default:
     * blocks that take part, and the phase work at or below which a phase
     * runs in block 0 alone (the result is the same for every shape) */
    int rl_blocks, rl_small;
    const int *rl_ptr, *rl_col, *sc_ptr, *sc_pos, *sc_piv;
    const int *ud_ptr, *ud_dst, *ud_cptr, *ud_l, *ud_u, *ud_p;  /* ud_p: pivot pos */
    /* the same schedule packed: per destination {lux pos, or -(pos + 1)
     * when it receives more than one product, the first product's L pos,
     * its U pos, the pivot k when the destination is U(k,k) and this is its
     * last update, else -1}, further products at ud_l/ud_u [ud_cptr[d] + 1
     * ..]; per L entry to scale {pos, its pivot's lux pos} (16- and 8-byte
     * aligned groups of ints, read as int4 / int2) */
    const int *ud_pk;
    const int *sc_pk;
    double *work;         /* [n] solve workspace */
    double *uinv;         /* [n] 1 / U(k,k), written by the refactorization */
    /* matrix cells / rhs rows with more than NGSF_HEAVY contributions
     * (heavy[]) are summed in chunks of NGSF_HCHUNK contributions: chunk c
     * belongs to heavy entry hch_cell[c]; hch_ptr[h] is entry h's first
     * chunk; hpart[c] holds the chunk's partial sum */
    int nhchunk;
    const int *hch_ptr, *hch_cell;
    double *hpart;

    /* Newton / integration state */
    double *states;       /* [4][nstates] ring of CKTstates[0..3] */
    double *rhs, *rhsOld; /* [n+1] */

    /* breakpoints */
    double *breaks;       /* [breakcap] */
    int breakcap;

    /* output: accepted points, time + values of probes */
    double *out;          /* [outcap][1 + nprobe] */
    const int *probe;     /* [nprobe] equation numbers */
    int nprobe, outcap;

    /* optional per-iteration capture of the stamped system (parity) */
    double *cap_lux;      /* [capmax][nlu] */
    double *cap_rhs;      /* [capmax][n+1] */
    double *cap_meta;     /* [capmax][4]: time, delta, mode, order */
    int capmax;

    /* saved control block of a run paused for a host re-pivot */
    void *ctlsave;
    /* operating-point stepping saves (OldRhsOld, OldCKTstate0) */
    double *opsave_rhs, *opsave_st;

    /* results written by the engine */
    int *result;          /* see NGSF_R_* */
    double *fresult;      /* see NGSF_F_* */
    ngsf_wide_t *wide;    /* set only for a wide (cooperative) launch */
    ngsf_pred_t pred;     /* learned Newton predictor (kind 0: off) */
    /* per-phase SM clock cycles of the circuit's block (NGSF_P_*), summed
     * over a run; null = not recorded */
    long long *prof;
    /* windowed runs: the transient stops (NGSF_HELD) at the first accepted
     * point at or after pause_at (+inf: runs to tstop); run_resume makes a
     * launch continue the saved run instead of starting a fresh one */
    double pause_at;
    int run_resume;
    /* synchronised runs (sharedspice GetSyncData): the time loop also
     * stops (NGSF_HELD) at the two points where the reference calls
     * sharedsync, so that the host can hand the step to the caller */
    int sync;
    /* transient re-pivot rules beyond the reference's zero pivot: the
     * retry after a Newton failure factors with new pivots (retry_repivot)
     * and, when tran_growth > 0, an L entry past it asks for new pivots */
    double tran_growth;
    int retry_repivot;
    /* triangular solves driven by row dependencies instead of level
     * barriers (same bits); 0 (default): level by level */
    int solve_sf;
} ngsf_ckt_t;

/* phases of the per-phase clock record */
enum {
    NGSF_P_LOAD, NGSF_P_GATHER, NGSF_P_FACTOR, NGSF_P_SOLVE, NGSF_P_CONV, NGSF_P_TRUNC,
    NGSF_P_TOTAL, NGSF_P_ITERS, NGSF_P_COUNT
};

/* integer results */
enum {
    NGSF_R_STATUS, NGSF_R_NPOINTS, NGSF_R_ACCEPTED, NGSF_R_REJECTED,
    NGSF_R_NUMITER, NGSF_R_TRANITER, NGSF_R_TIMEPTS, NGSF_R_NCAP,
    NGSF_R_OPITER, NGSF_R_BADPIVOT, NGSF_R_REORDERS, NGSF_R_GUESSES, NGSF_R_GUESS1,
    NGSF_R_FALLBACKS, NGSF_R_COUNT
};
/* floating results */
enum { NGSF_F_TIME, NGSF_F_DELTA, NGSF_F_DIAGGMIN, NGSF_F_COUNT };
/* internal results after the public ones: the sharedsync point a
 * synchronised run stopped at (0: none, 1 + the reference's loc), its
 * redostep, and the step's olddelta */
enum { NGSF_R_SYNCLOC = NGSF_R_COUNT, NGSF_R_SYNCREDO, NGSF_R_ALL };
enum { NGSF_F_OLDDELTA = NGSF_F_COUNT, NGSF_F_ALL };

#ifdef __cplusplus
}
#endif
#endif
