/*
 * Test infrastructure: CPU restatement of the reference transient path.
 * This is the oracle that the GPU engine is checked against on the GPU machine
 * (where the reference itself cannot be built) and the CPU baseline that
 * bench.py times.  Nothing in the product links or calls it.
 *
 * Restated, function by function, from the reference sources:
 *   port_run          DCtran, XSPICE variant   src/spicelib/analysis/dctran.c:67-971
 *   op_solve          CKTop + dynamic_gmin + new_gmin + gillespie_src
 *                                              src/spicelib/analysis/cktop.c:27-654
 *   ni_iter           NIiter                   src/maths/ni/niiter.c:29-367
 *   conv_test         NIconvTest + CKTconvTest src/maths/ni/niconv.c:21-90
 *   comcof            NIcomCof (trap, Gear 1-2) src/maths/ni/nicomcof.c:17-130
 *   integrate         NIintegrate (trap, Gear) src/maths/ni/niinteg.c:18-80
 *   terr / trunc      CKTterr / CKTtrunc       src/spicelib/analysis/cktterr.c:13-79,
 *                                              ckttrunc.c:20-57
 *   set_break/clr_break CKTsetBreak/CKTclrBreak src/spicelib/analysis/cktsetbk.c,
 *                                              cktclrbk.c
 *   src_value/src_accept VSRCload/VSRCaccept   src/spicelib/devices/vsrc/vsrcload.c,
 *                                              vsrcacct.c
 *   cap_load          CAPload                  src/spicelib/devices/cap/capload.c:15-87
 *   res_load          RESload                  src/spicelib/devices/res/resload.c:15-40
 *   mos1_load         MOS1load                 src/spicelib/devices/mos1/mos1load.c:17-941
 *   mos1_conv         MOS1convTest             src/spicelib/devices/mos1/mos1conv.c:13-99
 *   limvds/pnjlim/fetlim/qmeyer  devsup.c:21,50,93,674
 *   lu_*              dense LU with partial pivoting standing in for KLU
 *                     (klu_factor / klu_refactor / klu_solve): the pivot
 *                     sequence is chosen when the reference reorders and
 *                     reused otherwise.
 * The circuit arrives pre-compiled (node numbering, device order, and
 * temperature-dependent parameters) from oracle/port/port.py.
 *
 * Compile with floating-point contraction off (-ffp-contract=off) so that
 * x86-64 and Arm hosts evaluate every expression the same way.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAX(a, b) ((a) > (b) ? (a) : (b))
#define MIN(a, b) ((a) < (b) ? (a) : (b))

/* CKTmode bits (src/include/ngspice/cktdefs.h:171-199) */
#define MODETRAN 0x1
#define MODEDC 0x70
#define MODEDCOP 0x10
#define MODETRANOP 0x20
#define MODEDCTRANCURVE 0x40
#define INITF 0x3f00
#define MODEINITFLOAT 0x100
#define MODEINITJCT 0x200
#define MODEINITFIX 0x400
#define MODEINITSMSIG 0x800
#define MODEINITTRAN 0x1000
#define MODEINITPRED 0x2000
#define MODEUIC 0x10000

#define E_ITERLIM 101
#define E_SINGULAR 102
#define E_TIMESTEP 106
#define E_NOOP 110

/* MOS1 parameter and state layout: same order as the product's, but the
 * numbers are produced independently by port.py */
enum {
    P_TYPE, P_VT, P_DSAT, P_SSAT, P_CGSO, P_CGDO, P_CGBO, P_BETA, P_COX, P_TPHI,
    P_TVBI, P_TVTO, P_GAMMA, P_LAMBDA, P_SVCRIT, P_DVCRIT, P_CBS, P_CBSSW, P_CBD,
    P_CBDSW, P_TDEPCAP, P_TBULKPOT, P_F2S, P_F3S, P_F4S, P_F2D, P_F3D, P_F4D, P_MJ,
    P_MJSW, P_GDRAIN, P_GSOURCE, P_OFF, P_ICVDS, P_ICVGS, P_ICVBS, P_NPARAM
};
enum {
    S_VBD, S_VBS, S_VGS, S_VDS, S_CAPGS, S_QGS, S_CQGS, S_CAPGD, S_QGD, S_CQGD, S_CAPGB,
    S_QGB, S_CQGB, S_QBD, S_CQBD, S_QBS, S_CQBS
};

typedef struct {
    int node[6];        /* d g s b dp sp */
    int st;
    double p[P_NPARAM];
    /* instance memories */
    int mode;
    double von, vdsat, cd, cbs, cbd, gbs, gbd, gm, gds, gmbs, capbs, capbd;
} mos1_t;

/* BSIM4: parameters resolved and evaluated by the shared model arithmetic
 * (b4port.cpp); the port assembles the stamps in the reference order */
#define B4_MAXPARAM 256
#define B4_MAXSTAMP 64
typedef struct {
    int node[6];        /* d g s b dp sp */
    int st;
    double p[B4_MAXPARAM];
    double h[4];
} b4_t;
int port_b4_nparam(void);
int port_b4_nstamp(void);
void port_b4_pattern(int *rows, int *cols);
int port_b4_load_one(int mode, int order, int gear, double gmin, double delta,
                     double deltaOld1, double ag0, double ag1, double ag2, const double *rhsOld,
                     double *st0, double *st1, const double *st2, const double *p, double *h,
                     const int *node, int st, double *sv);

/* sparse mode for large circuits (sparse_port.cpp plans the pivots) */
typedef struct {
    int n, nnz, nlu, nlevels, nflevels, nblevels;
    int *a_lupos, *cdiag, *cend, *kptr, *kpos, *kseg, *upd_dst, *upd_src, *prow, *pcol;
    int *lvl_ptr, *lvl_col, *fl_ptr, *fl_row, *bl_ptr, *bl_row;
    int *lr_ptr, *lr_col, *lr_pos, *ur_ptr, *ur_col, *ur_pos;
    int nrl_levels, btf_blocks;   /* right-looking levels; KLU-order blocks */
    double flops;                 /* multiply-adds of one refactorization */
} port_plan_t;
int port_plan(int n, const int *cp, const int *ri, const double *ax, double pivrel,
              double pivtol, port_plan_t *out);
void port_plan_free(port_plan_t *p);

/* junction diode through the shared evaluation (b4port.cpp) */
#define DIO_MAXPARAM 64
typedef struct {
    int node[3];        /* pos neg pos' */
    int st;
    double p[DIO_MAXPARAM];
} dio_t;
int port_dio_nparam(void);
int port_dio_load_one(int mode, int order, int gear, double gmin, double delta,
                      double deltaOld1, double ag0, double ag1, double ag2, const double *rhsOld,
                      double *st0, double *st1, const double *st2, const double *p,
                      const int *node, int st, double *sv);

typedef struct { int a, b; double g; } res_t;
typedef struct { int a, b, st; double c, m, ic; } cap_t;
typedef struct {
    int p, n, br, kind, ncoef, dcgiven;
    double coef[64], dc, m, brk;
} src_t;

typedef struct {
    int n, nstates;
    int *ntype;
    /* devices in reference iteration order */
    int nres, ncap, nvsrc, nisrc, nmos1, nb4, ndio;
    res_t *res;
    cap_t *cap;
    src_t *vsrc, *isrc;
    mos1_t *mos1;
    b4_t *b4;
    dio_t *dio;
    /* options */
    double reltol, abstol, vntol, chgtol, trtol, gmin0, pivtol, pivrel, xmu;
    double tstep, tstop, tstart, tmax, delmin, minbreak;
    int itl1, itl4, maxord, method;   /* method: 0 trapezoidal, 1 Gear */
    /* run state */
    int sparse;              /* 1: CSC matrix + planned sparse LU */
    int recording, nrec, caprec, *rec;   /* pattern discovery (sparse) */
    int *cp, *ri, nnz;       /* CSC pattern, 0-based rows/cols */
    double *ax, *lux, *work, trash;
    port_plan_t plan;
    int havePlan;
    double *A, *LU;          /* dense (n+1)^2, row/col 0 = ground trash */
    int *perm;               /* row permutation of the factorization */
    int haveLU;
    double *rhs, *rhsOld, *states[4], *opsave_rhs, *opsave_st;
    double *breaks;
    int nbreaks, breakcap;
    double time, delta, deltaOld[7], ag[7], saveDelta;
    int order, mode, shouldReorder;
    double gmin, diagGmin, srcFact;
    long numIter, tranIter, timePts, accepted, rejected, opIter, reorders;
    /* output */
    double *out;
    int outcap, npoints;
    /* optional iteration dump */
    double *dump_ax, *dump_rhs, *dump_rhsold, *dump_meta;
    int dumpcap, ndump;
} port_t;

/* matrix element (r, k), 1-based; row or column 0 is the ground trash */
static double *port_elt(port_t *c, int r, int k)
{
    if (!c->sparse)
        return &c->A[(size_t)r * (c->n + 1) + k];
    if (r == 0 || k == 0)
        return &c->trash;
    if (c->recording) {
        if (c->nrec == c->caprec) {
            c->caprec = c->caprec ? 2 * c->caprec : 1024;
            c->rec = realloc(c->rec, sizeof(int) * 2 * (size_t)c->caprec);
        }
        c->rec[2 * c->nrec] = k - 1;
        c->rec[2 * c->nrec + 1] = r - 1;
        c->nrec++;
        return &c->trash;
    }
    int lo = c->cp[k - 1], hi = c->cp[k] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (c->ri[mid] < r - 1)
            lo = mid + 1;
        else if (c->ri[mid] > r - 1)
            hi = mid - 1;
        else
            return &c->ax[mid];
    }
    return &c->trash;   /* not reached: every stamped cell is in the pattern */
}
#define A_(c, r, k) (*port_elt((c), (r), (k)))

port_t *port_new(int n, int nstates)
{
    port_t *c = calloc(1, sizeof(port_t));
    c->n = n;
    c->nstates = nstates;
    c->ntype = calloc((size_t)n + 1, sizeof(int));
    c->sparse = n > 400;
    if (!c->sparse) {
        c->A = calloc((size_t)(n + 1) * (n + 1), sizeof(double));
        c->LU = calloc((size_t)(n + 1) * (n + 1), sizeof(double));
    } else {
        c->work = calloc((size_t)n + 1, sizeof(double));
    }
    c->perm = calloc((size_t)n + 1, sizeof(int));
    c->rhs = calloc((size_t)n + 1, sizeof(double));
    c->rhsOld = calloc((size_t)n + 1, sizeof(double));
    c->opsave_rhs = calloc((size_t)n + 1, sizeof(double));
    for (int i = 0; i < 4; i++)
        c->states[i] = calloc((size_t)nstates + 1, sizeof(double));
    c->opsave_st = calloc((size_t)nstates + 1, sizeof(double));
    return c;
}

void port_free(port_t *c)
{
    if (!c)
        return;
    free(c->ntype);
    free(c->A);
    free(c->LU);
    free(c->perm);
    free(c->rhs);
    free(c->rhsOld);
    free(c->opsave_rhs);
    free(c->opsave_st);
    for (int i = 0; i < 4; i++)
        free(c->states[i]);
    free(c->res);
    free(c->cap);
    free(c->vsrc);
    free(c->isrc);
    free(c->mos1);
    free(c->b4);
    free(c->dio);
    free(c->breaks);
    free(c->rec);
    free(c->cp);
    free(c->ri);
    free(c->ax);
    free(c->lux);
    free(c->work);
    port_plan_free(&c->plan);
    free(c);
}

void port_set_ntype(port_t *c, const int *t) { memcpy(c->ntype, t, sizeof(int) * (c->n + 1)); }

void port_set_options(port_t *c, const double *d, const int *i)
{
    c->reltol = d[0]; c->abstol = d[1]; c->vntol = d[2]; c->chgtol = d[3];
    c->trtol = d[4]; c->gmin0 = d[5]; c->pivtol = d[6]; c->pivrel = d[7];
    c->xmu = d[8]; c->tstep = d[9]; c->tstop = d[10]; c->tstart = d[11];
    c->tmax = d[12]; c->delmin = d[13]; c->minbreak = d[14];
    c->itl1 = i[0]; c->itl4 = i[1]; c->maxord = i[2]; c->method = i[3];
}

void port_add_res(port_t *c, int a, int b, double g)
{
    c->res = realloc(c->res, sizeof(res_t) * (c->nres + 1));
    c->res[c->nres++] = (res_t){a, b, g};
}

void port_add_cap(port_t *c, int a, int b, int st, double cval, double m, double ic)
{
    c->cap = realloc(c->cap, sizeof(cap_t) * (c->ncap + 1));
    c->cap[c->ncap++] = (cap_t){a, b, st, cval, m, ic};
}

void port_add_src(port_t *c, int isv, int p, int n, int br, int kind, int ncoef,
                  const double *coef, double dc, int dcgiven, double m)
{
    src_t s;
    memset(&s, 0, sizeof s);
    s.p = p; s.n = n; s.br = br; s.kind = kind; s.ncoef = ncoef;
    for (int k = 0; k < ncoef && k < 64; k++)
        s.coef[k] = coef[k];
    s.dc = dc; s.dcgiven = dcgiven; s.m = m;
    if (isv) {
        c->vsrc = realloc(c->vsrc, sizeof(src_t) * (c->nvsrc + 1));
        c->vsrc[c->nvsrc++] = s;
    } else {
        c->isrc = realloc(c->isrc, sizeof(src_t) * (c->nisrc + 1));
        c->isrc[c->nisrc++] = s;
    }
}

void port_add_mos1(port_t *c, const int *nodes, int st, const double *p)
{
    mos1_t m;
    memset(&m, 0, sizeof m);
    memcpy(m.node, nodes, sizeof m.node);
    m.st = st;
    memcpy(m.p, p, sizeof m.p);
    c->mos1 = realloc(c->mos1, sizeof(mos1_t) * (c->nmos1 + 1));
    c->mos1[c->nmos1++] = m;
}

void port_add_b4(port_t *c, const int *nodes, int st, const double *p)
{
    b4_t m;
    memset(&m, 0, sizeof m);
    memcpy(m.node, nodes, sizeof m.node);
    m.st = st;
    memcpy(m.p, p, sizeof(double) * port_b4_nparam());
    c->b4 = realloc(c->b4, sizeof(b4_t) * (c->nb4 + 1));
    c->b4[c->nb4++] = m;
}

void port_add_dio(port_t *c, const int *nodes, int st, const double *p)
{
    dio_t d;
    memset(&d, 0, sizeof d);
    memcpy(d.node, nodes, sizeof d.node);
    d.st = st;
    memcpy(d.p, p, sizeof(double) * port_dio_nparam());
    c->dio = realloc(c->dio, sizeof(dio_t) * (c->ndio + 1));
    c->dio[c->ndio++] = d;
}

void port_set_output(port_t *c, double *out, int outcap)
{
    c->out = out;
    c->outcap = outcap;
}

void port_set_dump(port_t *c, double *ax, double *rhs, double *rhsold, double *meta, int cap)
{
    c->dump_ax = ax; c->dump_rhs = rhs; c->dump_rhsold = rhsold; c->dump_meta = meta;
    c->dumpcap = cap;
}

/* ------------------------------------------------------------------ */
static int almost_equal_ulps(double a, double b, int maxUlps)
{
    int64_t ai, bi, d;
    if (a == b)
        return 1;
    memcpy(&ai, &a, 8);
    if (ai < 0)
        ai = INT64_MIN - ai;
    memcpy(&bi, &b, 8);
    if (bi < 0)
        bi = INT64_MIN - bi;
    d = ai - bi;
    if (d < 0)
        d = -d;
    return d <= maxUlps;
}

static double limvds(double vnew, double vold)
{
    if (vold >= 3.5) {
        if (vnew > vold)
            vnew = MIN(vnew, (3 * vold) + 2);
        else if (vnew < 3.5)
            vnew = MAX(vnew, 2);
    } else {
        if (vnew > vold)
            vnew = MIN(vnew, 4);
        else
            vnew = MAX(vnew, -.5);
    }
    return vnew;
}

static double pnjlim(double vnew, double vold, double vt, double vcrit, int *icheck)
{
    double arg;
    if ((vnew > vcrit) && (fabs(vnew - vold) > (vt + vt))) {
        if (vold > 0) {
            arg = (vnew - vold) / vt;
            if (arg > 0)
                vnew = vold + vt * (2 + log(arg - 2));
            else
                vnew = vold - vt * (2 + log(2 - arg));
        } else {
            vnew = vt * log(vnew / vt);
        }
        *icheck = 1;
    } else {
        if (vnew < 0) {
            if (vold > 0)
                arg = -1 * vold - 1;
            else
                arg = 2 * vold - 1;
            if (vnew < arg) {
                vnew = arg;
                *icheck = 1;
            } else {
                *icheck = 0;
            }
        } else {
            *icheck = 0;
        }
    }
    return vnew;
}

static double fetlim(double vnew, double vold, double vto)
{
    double vtsthi = fabs(2 * (vold - vto)) + 2;
    double vtstlo = fabs(vold - vto) + 1;
    double vtox = vto + 3.5;
    double delv = vnew - vold;
    if (vold >= vto) {
        if (vold >= vtox) {
            if (delv <= 0) {
                if (vnew >= vtox) {
                    if (-delv > vtstlo)
                        vnew = vold - vtstlo;
                } else {
                    vnew = MAX(vnew, vto + 2);
                }
            } else if (delv >= vtsthi) {
                vnew = vold + vtsthi;
            }
        } else if (delv <= 0) {
            vnew = MAX(vnew, vto - .5);
        } else {
            vnew = MIN(vnew, vto + 4);
        }
    } else if (delv <= 0) {
        if (-delv > vtsthi)
            vnew = vold - vtsthi;
    } else {
        double vtemp = vto + .5;
        if (vnew <= vtemp) {
            if (delv > vtstlo)
                vnew = vold + vtstlo;
        } else {
            vnew = vtemp;
        }
    }
    return vnew;
}

static void qmeyer(double vgs, double vgd, double von, double vdsat, double *capgs,
                   double *capgd, double *capgb, double phi, double cox)
{
    double vds, vddif, vddif1, vddif2, vgst;
    vgst = vgs - von;
    vdsat = MAX(vdsat, 0.025);
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
        vds = vgs - vgd;
        if (vds >= vdsat) {
            *capgd = 0;
        } else {
            vddif = 2.0 * vdsat - vds;
            vddif1 = vdsat - vds;
            vddif2 = vddif * vddif;
            *capgd = *capgs * (1.0 - vdsat * vdsat / vddif2);
            *capgs = *capgs * (1.0 - vddif1 * vddif1 / vddif2);
        }
    } else {
        vds = vgs - vgd;
        vdsat = MAX(vdsat, 0.025);
        if (vdsat <= vds) {
            *capgs = cox / 3;
            *capgd = 0;
            *capgb = 0;
        } else {
            vddif = 2.0 * vdsat - vds;
            vddif1 = vdsat - vds;
            vddif2 = vddif * vddif;
            *capgd = cox * (1.0 - vdsat * vdsat / vddif2) / 3;
            *capgs = cox * (1.0 - vddif1 * vddif1 / vddif2) / 3;
            *capgb = 0;
        }
    }
}

static void integrate(port_t *c, double *geq, double *ceq, double cap, int qcap)
{
    double *s0 = c->states[0], *s1 = c->states[1], *s2 = c->states[2];
    int ccap = qcap + 1;
    if (c->method == 1) {
        /* Gear: sum of ag[k] * q_k, highest k first (niinteg.c:42-67) */
        s0[ccap] = 0;
        if (c->order >= 2)
            s0[ccap] += c->ag[2] * s2[qcap];
        s0[ccap] += c->ag[1] * s1[qcap];
        s0[ccap] += c->ag[0] * s0[qcap];
    } else if (c->order == 1)
        s0[ccap] = c->ag[0] * s0[qcap] + c->ag[1] * s1[qcap];
    else
        s0[ccap] = -s1[ccap] * c->ag[1] + c->ag[0] * (s0[qcap] - s1[qcap]);
    *ceq = s0[ccap] - c->ag[0] * s0[qcap];
    *geq = c->ag[0] * cap;
}

/* ------------------------------------------------------------------ */
/* device loads                                                        */
/* ------------------------------------------------------------------ */
static void cap_load(port_t *c)
{
    int mode = c->mode;
    double *s0 = c->states[0], *s1 = c->states[1];
    if (!(mode & (MODETRAN | MODETRANOP)))
        return;
    int cond1 = ((mode & MODEDC) && (mode & MODEINITJCT)) ||
                ((mode & MODEUIC) && (mode & MODEINITTRAN));
    for (int i = 0; i < c->ncap; i++) {
        cap_t *h = &c->cap[i];
        double vcap = cond1 ? h->ic : c->rhsOld[h->a] - c->rhsOld[h->b];
        if (mode & MODETRAN) {
            double geq, ceq;
            if (mode & MODEINITPRED) {
                s0[h->st] = s1[h->st];
            } else {
                s0[h->st] = h->c * vcap;
                if (mode & MODEINITTRAN)
                    s1[h->st] = s0[h->st];
            }
            integrate(c, &geq, &ceq, h->c, h->st);
            if (mode & MODEINITTRAN)
                s1[h->st + 1] = s0[h->st + 1];
            A_(c, h->a, h->a) += h->m * geq;
            A_(c, h->b, h->b) += h->m * geq;
            A_(c, h->a, h->b) -= h->m * geq;
            A_(c, h->b, h->a) -= h->m * geq;
            c->rhs[h->a] -= h->m * ceq;
            c->rhs[h->b] += h->m * ceq;
        } else {
            s0[h->st] = h->c * vcap;
        }
    }
}

static double src_value(port_t *c, const src_t *h)
{
    int mode = c->mode;
    if ((mode & (MODEDCOP | MODEDCTRANCURVE)) && h->dcgiven)
        return h->dc;
    double time = (mode & MODEDC) ? 0.0 : c->time;
    const double *cf = h->coef;
    int nc = h->ncoef;
    double value = 0;
    switch (h->kind) {
    default:
        value = h->dc;
        break;
    case 1: { /* PULSE */
        double V1 = cf[0], V2 = cf[1];
        double TD = nc > 2 ? cf[2] : 0.0;
        double TR = nc > 3 && cf[3] > 0.0 ? cf[3] : c->tstep;
        double TF = nc > 4 && cf[4] > 0.0 ? cf[4] : c->tstep;
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
            if (time > PER)
                time -= PER * floor(time / PER);
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
    case 2: { /* SIN */
        double PHASE = nc > 5 ? cf[5] : 0.0;
        double phase = PHASE * M_PI / 180.0;
        double VO = cf[0], VA = cf[1];
        double FREQ = nc > 2 && cf[2] != 0.0 ? cf[2] : (1 / c->tstop);
        double TD = nc > 3 ? cf[3] : 0.0;
        double THETA = nc > 4 ? cf[4] : 0.0;
        time -= TD;
        if (time <= 0)
            value = VO + VA * sin(phase);
        else
            value = VO + VA * sin(FREQ * time * 2.0 * M_PI + phase) * exp(-time * THETA);
        break;
    }
    case 4: { /* PWL */
        if (time <= cf[0]) {
            value = cf[1];
            break;
        }
        if (time > cf[nc - 2]) {
            value = cf[nc - 1];
            break;
        }
        for (int k = 2; k < nc; k += 2) {
            if (cf[k] >= time) {
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
    if (mode & MODETRANOP)
        value *= c->srcFact;
    return value;
}

static void src_load(port_t *c)
{
    for (int i = 0; i < c->nisrc; i++) {
        src_t *h = &c->isrc[i];
        double v = src_value(c, h);
        c->rhs[h->p] += h->m * v;
        c->rhs[h->n] -= h->m * v;
    }
}

static void vsrc_load(port_t *c)
{
    for (int i = 0; i < c->nvsrc; i++) {
        src_t *h = &c->vsrc[i];
        A_(c, h->p, h->br) += 1.0;
        A_(c, h->n, h->br) -= 1.0;
        A_(c, h->br, h->p) += 1.0;
        A_(c, h->br, h->n) -= 1.0;
        c->rhs[h->br] += src_value(c, h);
    }
}

static void res_load(port_t *c)
{
    for (int i = 0; i < c->nres; i++) {
        res_t *h = &c->res[i];
        A_(c, h->a, h->a) += h->g;
        A_(c, h->b, h->b) += h->g;
        A_(c, h->a, h->b) -= h->g;
        A_(c, h->b, h->a) -= h->g;
    }
}

static int mos1_load(port_t *c)
{
    int noncon = 0;
    int mode = c->mode;
    double *s0 = c->states[0], *s1 = c->states[1], *s2 = c->states[2];
    for (int ii = 0; ii < c->nmos1; ii++) {
        mos1_t *h = &c->mos1[ii];
        const double *p = h->p;
        double *st0 = s0 + h->st, *st1 = s1 + h->st, *st2 = s2 + h->st;
        int dN = h->node[0], gN = h->node[1], sN = h->node[2], bN = h->node[3];
        int dpN = h->node[4], spN = h->node[5];
        double type = p[P_TYPE], vt = p[P_VT];
        int off = p[P_OFF] != 0.0;
        int Check = 1;
        double xfact = 0, vbs, vgs, vds, vbd, vgd, vgb, von, vdsat;
        double cdrain, capgs = 0, capgd = 0, capgb = 0;
        if ((mode & (MODEINITFLOAT | MODEINITPRED | MODEINITSMSIG | MODEINITTRAN)) ||
            ((mode & MODEINITFIX) && !off)) {
            if (mode & (MODEINITPRED | MODEINITTRAN)) {
                xfact = c->delta / c->deltaOld[1];
                st0[S_VBS] = st1[S_VBS];
                vbs = (1 + xfact) * (st1[S_VBS]) - (xfact * (st2[S_VBS]));
                st0[S_VGS] = st1[S_VGS];
                vgs = (1 + xfact) * (st1[S_VGS]) - (xfact * (st2[S_VGS]));
                st0[S_VDS] = st1[S_VDS];
                vds = (1 + xfact) * (st1[S_VDS]) - (xfact * (st2[S_VDS]));
                st0[S_VBD] = st0[S_VBS] - st0[S_VDS];
            } else {
                vbs = type * (c->rhsOld[bN] - c->rhsOld[spN]);
                vgs = type * (c->rhsOld[gN] - c->rhsOld[spN]);
                vds = type * (c->rhsOld[dpN] - c->rhsOld[spN]);
            }
            vbd = vbs - vds;
            vgd = vgs - vds;
            double vgdo = st0[S_VGS] - st0[S_VDS];
            von = type * h->von;
            if (st0[S_VDS] >= 0) {
                vgs = fetlim(vgs, st0[S_VGS], von);
                vds = vgs - vgd;
                vds = limvds(vds, st0[S_VDS]);
                vgd = vgs - vds;
            } else {
                vgd = fetlim(vgd, vgdo, von);
                vds = vgs - vgd;
                vds = -limvds(-vds, -(st0[S_VDS]));
                vgs = vgd + vds;
            }
            if (vds >= 0) {
                vbs = pnjlim(vbs, st0[S_VBS], vt, p[P_SVCRIT], &Check);
                vbd = vbs - vds;
            } else {
                vbd = pnjlim(vbd, st0[S_VBD], vt, p[P_DVCRIT], &Check);
                vbs = vbd + vds;
            }
        } else {
            if ((mode & MODEINITJCT) && !off) {
                vds = type * p[P_ICVDS];
                vgs = type * p[P_ICVGS];
                vbs = type * p[P_ICVBS];
                if ((vds == 0) && (vgs == 0) && (vbs == 0) &&
                    ((mode & (MODETRAN | MODEDCOP | MODEDCTRANCURVE)) || (!(mode & MODEUIC)))) {
                    vbs = -1;
                    vgs = type * p[P_TVTO];
                    vds = 0;
                }
            } else {
                vbs = vgs = vds = 0;
            }
        }
        vbd = vbs - vds;
        vgd = vgs - vds;
        vgb = vgs - vbs;
        if (vbs <= -3 * vt) {
            h->gbs = c->gmin;
            h->cbs = h->gbs * vbs - p[P_SSAT];
        } else {
            double evbs = exp(MIN(709.0, vbs / vt));
            h->gbs = p[P_SSAT] * evbs / vt + c->gmin;
            h->cbs = p[P_SSAT] * (evbs - 1) + c->gmin * vbs;
        }
        if (vbd <= -3 * vt) {
            h->gbd = c->gmin;
            h->cbd = h->gbd * vbd - p[P_DSAT];
        } else {
            double evbd = exp(MIN(709.0, vbd / vt));
            h->gbd = p[P_DSAT] * evbd / vt + c->gmin;
            h->cbd = p[P_DSAT] * (evbd - 1) + c->gmin * vbd;
        }
        h->mode = vds >= 0 ? 1 : -1;
        {
            double arg, betap, sarg, vgst;
            double vbx = h->mode == 1 ? vbs : vbd;
            if (vbx <= 0) {
                sarg = sqrt(p[P_TPHI] - vbx);
            } else {
                sarg = sqrt(p[P_TPHI]);
                sarg = sarg - vbx / (sarg + sarg);
                sarg = MAX(0, sarg);
            }
            von = (p[P_TVBI] * type) + p[P_GAMMA] * sarg;
            vgst = (h->mode == 1 ? vgs : vgd) - von;
            vdsat = MAX(vgst, 0);
            arg = sarg <= 0 ? 0 : p[P_GAMMA] / (sarg + sarg);
            if (vgst <= 0) {
                cdrain = 0;
                h->gm = 0;
                h->gds = 0;
                h->gmbs = 0;
            } else {
                betap = p[P_BETA] * (1 + p[P_LAMBDA] * (vds * h->mode));
                if (vgst <= (vds * h->mode)) {
                    cdrain = betap * vgst * vgst * .5;
                    h->gm = betap * vgst;
                    h->gds = p[P_LAMBDA] * p[P_BETA] * vgst * vgst * .5;
                    h->gmbs = h->gm * arg;
                } else {
                    cdrain = betap * (vds * h->mode) * (vgst - .5 * (vds * h->mode));
                    h->gm = betap * (vds * h->mode);
                    h->gds = betap * (vgst - (vds * h->mode)) +
                             p[P_LAMBDA] * p[P_BETA] * (vds * h->mode) *
                                 (vgst - .5 * (vds * h->mode));
                    h->gmbs = h->gm * arg;
                }
            }
        }
        h->von = type * von;
        h->vdsat = type * vdsat;
        h->cd = h->mode * cdrain - h->cbd;
        if (mode & (MODETRAN | MODETRANOP | MODEINITSMSIG)) {
            double mj = p[P_MJ], mjsw = p[P_MJSW], pb = p[P_TBULKPOT];
            if (p[P_CBS] != 0 || p[P_CBSSW] != 0) {
                if (vbs < p[P_TDEPCAP]) {
                    double arg = 1 - vbs / pb, sarg, sargsw;
                    if (mj == mjsw) {
                        if (mj == .5)
                            sarg = sargsw = 1 / sqrt(arg);
                        else
                            sarg = sargsw = exp(-mj * log(arg));
                    } else {
                        sarg = mj == .5 ? 1 / sqrt(arg) : exp(-mj * log(arg));
                        sargsw = mjsw == .5 ? 1 / sqrt(arg) : exp(-mjsw * log(arg));
                    }
                    st0[S_QBS] = pb * (p[P_CBS] * (1 - arg * sarg) / (1 - mj) +
                                       p[P_CBSSW] * (1 - arg * sargsw) / (1 - mjsw));
                    h->capbs = p[P_CBS] * sarg + p[P_CBSSW] * sargsw;
                } else {
                    st0[S_QBS] = p[P_F4S] + vbs * (p[P_F2S] + vbs * (p[P_F3S] / 2));
                    h->capbs = p[P_F2S] + p[P_F3S] * vbs;
                }
            } else {
                st0[S_QBS] = 0;
                h->capbs = 0;
            }
            if (p[P_CBD] != 0 || p[P_CBDSW] != 0) {
                if (vbd < p[P_TDEPCAP]) {
                    double arg = 1 - vbd / pb, sarg, sargsw;
                    if (mj == .5 && mjsw == .5) {
                        sarg = sargsw = 1 / sqrt(arg);
                    } else {
                        sarg = mj == .5 ? 1 / sqrt(arg) : exp(-mj * log(arg));
                        sargsw = mjsw == .5 ? 1 / sqrt(arg) : exp(-mjsw * log(arg));
                    }
                    st0[S_QBD] = pb * (p[P_CBD] * (1 - arg * sarg) / (1 - mj) +
                                       p[P_CBDSW] * (1 - arg * sargsw) / (1 - mjsw));
                    h->capbd = p[P_CBD] * sarg + p[P_CBDSW] * sargsw;
                } else {
                    st0[S_QBD] = p[P_F4D] + vbd * (p[P_F2D] + vbd * p[P_F3D] / 2);
                    h->capbd = p[P_F2D] + vbd * p[P_F3D];
                }
            } else {
                st0[S_QBD] = 0;
                h->capbd = 0;
            }
            if ((mode & MODETRAN) || ((mode & MODEINITTRAN) && !(mode & MODEUIC))) {
                double geq, ceq;
                integrate(c, &geq, &ceq, h->capbd, h->st + S_QBD);
                h->gbd += geq;
                h->cbd += st0[S_CQBD];
                h->cd -= st0[S_CQBD];
                integrate(c, &geq, &ceq, h->capbs, h->st + S_QBS);
                h->gbs += geq;
                h->cbs += st0[S_CQBS];
            }
        }
        if (!off || !(mode & (MODEINITFIX | MODEINITSMSIG)))
            if (Check == 1)
                noncon++;
        st0[S_VBS] = vbs;
        st0[S_VBD] = vbd;
        st0[S_VGS] = vgs;
        st0[S_VDS] = vds;
        if (mode & (MODETRAN | MODETRANOP | MODEINITSMSIG)) {
            if (h->mode > 0)
                qmeyer(vgs, vgd, von, vdsat, &st0[S_CAPGS], &st0[S_CAPGD], &st0[S_CAPGB],
                       p[P_TPHI], p[P_COX]);
            else
                qmeyer(vgd, vgs, von, vdsat, &st0[S_CAPGD], &st0[S_CAPGS], &st0[S_CAPGB],
                       p[P_TPHI], p[P_COX]);
            double vgs1 = st1[S_VGS], vgd1 = vgs1 - st1[S_VDS], vgb1 = vgs1 - st1[S_VBS];
            if (mode & (MODETRANOP | MODEINITSMSIG)) {
                capgs = 2 * st0[S_CAPGS] + p[P_CGSO];
                capgd = 2 * st0[S_CAPGD] + p[P_CGDO];
                capgb = 2 * st0[S_CAPGB] + p[P_CGBO];
            } else {
                capgs = (st0[S_CAPGS] + st1[S_CAPGS] + p[P_CGSO]);
                capgd = (st0[S_CAPGD] + st1[S_CAPGD] + p[P_CGDO]);
                capgb = (st0[S_CAPGB] + st1[S_CAPGB] + p[P_CGBO]);
            }
            if (mode & (MODEINITPRED | MODEINITTRAN)) {
                st0[S_QGS] = (1 + xfact) * st1[S_QGS] - xfact * st2[S_QGS];
                st0[S_QGD] = (1 + xfact) * st1[S_QGD] - xfact * st2[S_QGD];
                st0[S_QGB] = (1 + xfact) * st1[S_QGB] - xfact * st2[S_QGB];
            } else if (mode & MODETRAN) {
                st0[S_QGS] = (vgs - vgs1) * capgs + st1[S_QGS];
                st0[S_QGD] = (vgd - vgd1) * capgd + st1[S_QGD];
                st0[S_QGB] = (vgb - vgb1) * capgb + st1[S_QGB];
            } else {
                st0[S_QGS] = vgs * capgs;
                st0[S_QGD] = vgd * capgd;
                st0[S_QGB] = vgb * capgb;
            }
        }
        double gcgs, ceqgs, gcgd, ceqgd, gcgb, ceqgb;
        if ((mode & MODEINITTRAN) || !(mode & MODETRAN)) {
            gcgs = ceqgs = gcgd = ceqgd = gcgb = ceqgb = 0;
        } else {
            if (capgs == 0)
                st0[S_CQGS] = 0;
            if (capgd == 0)
                st0[S_CQGD] = 0;
            if (capgb == 0)
                st0[S_CQGB] = 0;
            integrate(c, &gcgs, &ceqgs, capgs, h->st + S_QGS);
            integrate(c, &gcgd, &ceqgd, capgd, h->st + S_QGD);
            integrate(c, &gcgb, &ceqgb, capgb, h->st + S_QGB);
            ceqgs = ceqgs - gcgs * vgs + c->ag[0] * st0[S_QGS];
            ceqgd = ceqgd - gcgd * vgd + c->ag[0] * st0[S_QGD];
            ceqgb = ceqgb - gcgb * vgb + c->ag[0] * st0[S_QGB];
        }
        double ceqbs = type * (h->cbs - (h->gbs) * vbs);
        double ceqbd = type * (h->cbd - (h->gbd) * vbd);
        double xnrm, xrev, cdreq;
        if (h->mode >= 0) {
            xnrm = 1;
            xrev = 0;
            cdreq = type * (cdrain - h->gds * vds - h->gm * vgs - h->gmbs * vbs);
        } else {
            xnrm = 0;
            xrev = 1;
            cdreq = -(type) * (cdrain - h->gds * (-vds) - h->gm * vgd - h->gmbs * vbd);
        }
        double gd = p[P_GDRAIN], gs = p[P_GSOURCE];
        c->rhs[gN] -= (type * (ceqgs + ceqgb + ceqgd));
        c->rhs[bN] -= (ceqbs + ceqbd - type * ceqgb);
        c->rhs[dpN] += (ceqbd - cdreq + type * ceqgd);
        c->rhs[spN] += cdreq + ceqbs + type * ceqgs;
        A_(c, dN, dN) += gd;
        A_(c, gN, gN) += gcgd + gcgs + gcgb;
        A_(c, sN, sN) += gs;
        A_(c, bN, bN) += h->gbd + h->gbs + gcgb;
        A_(c, dpN, dpN) += gd + h->gds + h->gbd + xrev * (h->gm + h->gmbs) + gcgd;
        A_(c, spN, spN) += gs + h->gds + h->gbs + xnrm * (h->gm + h->gmbs) + gcgs;
        A_(c, dN, dpN) += -gd;
        A_(c, gN, bN) -= gcgb;
        A_(c, gN, dpN) -= gcgd;
        A_(c, gN, spN) -= gcgs;
        A_(c, sN, spN) += -gs;
        A_(c, bN, gN) -= gcgb;
        A_(c, bN, dpN) -= h->gbd;
        A_(c, bN, spN) -= h->gbs;
        A_(c, dpN, dN) += -gd;
        A_(c, dpN, gN) += (xnrm - xrev) * h->gm - gcgd;
        A_(c, dpN, bN) += -h->gbd + (xnrm - xrev) * h->gmbs;
        A_(c, dpN, spN) += -h->gds - xnrm * (h->gm + h->gmbs);
        A_(c, spN, gN) += -(xnrm - xrev) * h->gm - gcgs;
        A_(c, spN, sN) += -gs;
        A_(c, spN, bN) += -h->gbs - (xnrm - xrev) * h->gmbs;
        A_(c, spN, dpN) += -h->gds - xrev * (h->gm + h->gmbs);
    }
    return noncon;
}

static int mos1_conv(port_t *c)
{
    double *s0 = c->states[0];
    for (int ii = 0; ii < c->nmos1; ii++) {
        mos1_t *h = &c->mos1[ii];
        double type = h->p[P_TYPE], *st0 = s0 + h->st;
        double vbs = type * (c->rhs[h->node[3]] - c->rhs[h->node[5]]);
        double vgs = type * (c->rhs[h->node[1]] - c->rhs[h->node[5]]);
        double vds = type * (c->rhs[h->node[4]] - c->rhs[h->node[5]]);
        double vbd = vbs - vds, vgd = vgs - vds;
        double vgdo = st0[S_VGS] - st0[S_VDS];
        double delvbs = vbs - st0[S_VBS], delvbd = vbd - st0[S_VBD];
        double delvgs = vgs - st0[S_VGS], delvds = vds - st0[S_VDS];
        double delvgd = vgd - vgdo, cdhat, cbhat, tol;
        if (h->mode >= 0)
            cdhat = h->cd - h->gbd * delvbd + h->gmbs * delvbs + h->gm * delvgs +
                    h->gds * delvds;
        else
            cdhat = h->cd - (h->gbd - h->gmbs) * delvbd - h->gm * delvgd + h->gds * delvds;
        cbhat = h->cbs + h->cbd + h->gbd * delvbd + h->gbs * delvbs;
        tol = c->reltol * MAX(fabs(cdhat), fabs(h->cd)) + c->abstol;
        if (fabs(cdhat - h->cd) >= tol)
            return 1;
        tol = c->reltol * MAX(fabs(cbhat), fabs(h->cbs + h->cbd)) + c->abstol;
        if (fabs(cbhat - (h->cbs + h->cbd)) > tol)
            return 1;
    }
    return 0;
}

/* BSIM4load + BSIM4LoadRhsMat (src/spicelib/devices/bsim4/b4ld.c:70-5623):
 * per instance, its right-hand-side terms and then its matrix terms */
static int b4_load(port_t *c)
{
    int nc = 0;
    static int rows[B4_MAXSTAMP], cols[B4_MAXSTAMP], ns = -1;
    if (ns < 0) {
        port_b4_pattern(rows, cols);
        ns = port_b4_nstamp();
    }
    double sv[B4_MAXSTAMP];
    for (int i = 0; i < c->nb4; i++) {
        b4_t *h = &c->b4[i];
        nc |= port_b4_load_one(c->mode, c->order, c->method, c->gmin, c->delta, c->deltaOld[1],
                               c->ag[0], c->ag[1], c->ag[2], c->rhsOld, c->states[0],
                               c->states[1], c->states[2],
                               h->p, h->h, h->node, h->st, sv);
        for (int k = 0; k < ns; k++) {
            if (rows[k] < 0)
                c->rhs[h->node[cols[k]]] += sv[k];
            else
                A_(c, h->node[rows[k]], h->node[cols[k]]) += sv[k];
        }
    }
    c->rhs[0] = 0.0;
    return nc;
}

static int ckt_load_devices(port_t *c);

static int cmp_pair(const void *a, const void *b)
{
    const int *x = a, *y = b;
    if (x[0] != y[0])
        return x[0] < y[0] ? -1 : 1;
    return x[1] < y[1] ? -1 : (x[1] > y[1]);
}

/* sparse mode: discover the matrix pattern from one recording load
 * (every element a device touches), then keep it for the run */
static void build_pattern(port_t *c)
{
    int n = c->n;
    c->recording = 1;
    c->nrec = 0;
    ckt_load_devices(c);
    c->recording = 0;
    for (int j = 0; j < n; j++) {      /* every equation keeps its diagonal */
        if (c->nrec == c->caprec) {
            c->caprec = c->caprec ? 2 * c->caprec : 1024;
            c->rec = realloc(c->rec, sizeof(int) * 2 * (size_t)c->caprec);
        }
        c->rec[2 * c->nrec] = j;
        c->rec[2 * c->nrec + 1] = j;
        c->nrec++;
    }
    qsort(c->rec, (size_t)c->nrec, 2 * sizeof(int), cmp_pair);
    c->cp = calloc((size_t)n + 1, sizeof(int));
    c->ri = malloc(sizeof(int) * (size_t)c->nrec);
    int m = 0;
    for (int t = 0; t < c->nrec; t++) {
        if (t && c->rec[2 * t] == c->rec[2 * t - 2] && c->rec[2 * t + 1] == c->rec[2 * t - 1])
            continue;
        c->ri[m++] = c->rec[2 * t + 1];
        c->cp[c->rec[2 * t] + 1]++;
    }
    for (int j = 0; j < n; j++)
        c->cp[j + 1] += c->cp[j];
    c->nnz = m;
    c->ax = calloc((size_t)m, sizeof(double));
}

/* DIOload (src/spicelib/devices/dio/dioload.c:785-815 stamp order) */
static int dio_load(port_t *c)
{
    int nc = 0;
    double sv[9];
    for (int i = 0; i < c->ndio; i++) {
        dio_t *d = &c->dio[i];
        nc |= port_dio_load_one(c->mode, c->order, c->method, c->gmin, c->delta, c->deltaOld[1],
                                c->ag[0], c->ag[1], c->ag[2], c->rhsOld, c->states[0],
                                c->states[1], c->states[2],
                                d->p, d->node, d->st, sv);
        int P = d->node[0], N = d->node[1], PP = d->node[2];
        c->rhs[N] += sv[0];
        c->rhs[PP] += sv[1];
        A_(c, P, P) += sv[2];
        A_(c, N, N) += sv[3];
        A_(c, PP, PP) += sv[4];
        A_(c, P, PP) += sv[5];
        A_(c, N, PP) += sv[6];
        A_(c, PP, P) += sv[7];
        A_(c, PP, N) += sv[8];
    }
    return nc;
}

static int ckt_load(port_t *c)
{
    int n = c->n;
    if (c->sparse && !c->cp) {
        /* the recording pass has the load's side effects (states of the
         * first iteration); the real pass below repeats them identically */
        memset(c->rhs, 0, sizeof(double) * (n + 1));
        build_pattern(c);
    }
    memset(c->rhs, 0, sizeof(double) * (n + 1));
    if (c->sparse)
        memset(c->ax, 0, sizeof(double) * (size_t)c->nnz);
    else
        memset(c->A, 0, sizeof(double) * (size_t)(n + 1) * (n + 1));
    return ckt_load_devices(c);
}

static int ckt_load_devices(port_t *c)
{
    /* reference device-table order: bsim4, cap, dio, isrc, mos1, res, vsrc */
    int nc = b4_load(c);
    cap_load(c);
    nc |= dio_load(c);
    src_load(c);
    nc |= mos1_load(c);
    res_load(c);
    vsrc_load(c);
    return nc;
}

/* ------------------------------------------------------------------ */
/* dense LU standing in for KLU: pivoting factorization when the        */
/* reference reorders, refactorization on the same pivots otherwise     */
/* ------------------------------------------------------------------ */
/* sparse refactorization on the planned pattern: left-looking, columns
 * in dependency-level order; fails (asking for new pivots) on a zero or
 * non-finite pivot or a non-finite L entry, and in the operating point
 * (MODEDCOP / MODETRANOP, where gmin and source stepping move the matrix
 * far from the one the pivots were chosen on) also on an L entry above
 * 1e6.  The transient refactors on its pivots like klu_refactor
 * (src/maths/KLU/klusmp.c:591-602: only a zero pivot fails); the retry
 * after a Newton failure re-pivots (port_run). */
static int sp_factor(port_t *c)
{
    port_plan_t *P = &c->plan;
    int n = c->n;
    const double growth = (c->mode & (MODEDCOP | MODETRANOP)) ? 1e6 : DBL_MAX;
    double *lux = c->lux;
    memset(lux, 0, sizeof(double) * (size_t)P->nlu);
    for (int p = 0; p < c->nnz; p++)
        lux[P->a_lupos[p]] = c->ax[p];
    if (c->diagGmin != 0)
        for (int j = 0; j < n; j++)
            for (int p = c->cp[j]; p < c->cp[j + 1]; p++)
                if (c->ri[p] == j)
                    lux[P->a_lupos[p]] += c->diagGmin;
    for (int l = 0; l < P->nlevels; l++)
        for (int q = P->lvl_ptr[l]; q < P->lvl_ptr[l + 1]; q++) {
            int k = P->lvl_col[q];
            for (int t = P->kptr[k]; t < P->kptr[k + 1]; t++) {
                double xk = lux[P->kpos[t]];
                for (int u = P->kseg[t]; u < P->kseg[t + 1]; u++)
                    lux[P->upd_dst[u]] -= lux[P->upd_src[u]] * xk;
            }
            double piv = lux[P->cdiag[k]];
            if (!(fabs(piv) > 0.0) || !isfinite(piv))
                return E_SINGULAR;
            for (int q2 = P->cdiag[k] + 1; q2 < P->cend[k]; q2++) {
                double lik = lux[q2] / piv;
                lux[q2] = lik;
                if (!(fabs(lik) <= growth))
                    return E_SINGULAR;
            }
        }
    return 0;
}

static int lu_factor(port_t *c, int repivot)
{
    int n = c->n;
    if (c->sparse) {
        if (repivot || !c->havePlan) {
            double *a = malloc(sizeof(double) * (size_t)c->nnz);
            memcpy(a, c->ax, sizeof(double) * (size_t)c->nnz);
            if (c->diagGmin != 0)
                for (int j = 0; j < n; j++)
                    for (int p = c->cp[j]; p < c->cp[j + 1]; p++)
                        if (c->ri[p] == j)
                            a[p] += c->diagGmin;
            int rc = port_plan(n, c->cp, c->ri, a, c->pivrel, c->pivtol, &c->plan);
            free(a);
            if (rc != 0)
                return E_SINGULAR;
            c->havePlan = 1;
            free(c->lux);
            c->lux = malloc(sizeof(double) * (size_t)c->plan.nlu);
        }
        return sp_factor(c);
    }
    double *L = c->LU;
    for (int r = 1; r <= n; r++)
        for (int k = 1; k <= n; k++)
            L[(size_t)r * (n + 1) + k] = A_(c, r, k);
    if (c->diagGmin != 0)
        for (int r = 1; r <= n; r++)
            L[(size_t)r * (n + 1) + r] += c->diagGmin;
    if (repivot || !c->haveLU) {
        for (int i = 1; i <= n; i++)
            c->perm[i] = i;
    }
    /* row-permuted copy */
    double *P = malloc(sizeof(double) * (size_t)(n + 1) * (n + 1));
    for (int i = 1; i <= n; i++)
        memcpy(P + (size_t)i * (n + 1), L + (size_t)c->perm[i] * (n + 1), sizeof(double) * (n + 1));
    for (int k = 1; k <= n; k++) {
        if (repivot || !c->haveLU) {
            int best = k;
            double bv = fabs(P[(size_t)k * (n + 1) + k]);
            for (int i = k + 1; i <= n; i++) {
                double v = fabs(P[(size_t)i * (n + 1) + k]);
                if (v > bv) {
                    bv = v;
                    best = i;
                }
            }
            /* threshold partial pivoting: keep the diagonal when it is
             * within pivrel of the column maximum */
            if (fabs(P[(size_t)k * (n + 1) + k]) >= c->pivrel * bv && fabs(P[(size_t)k * (n + 1) + k]) > 0)
                best = k;
            if (best != k) {
                for (int j = 0; j <= n; j++) {
                    double t = P[(size_t)k * (n + 1) + j];
                    P[(size_t)k * (n + 1) + j] = P[(size_t)best * (n + 1) + j];
                    P[(size_t)best * (n + 1) + j] = t;
                }
                int t = c->perm[k];
                c->perm[k] = c->perm[best];
                c->perm[best] = t;
            }
        }
        double d = P[(size_t)k * (n + 1) + k];
        if (!(fabs(d) > 0) || !isfinite(d)) {
            free(P);
            return E_SINGULAR;
        }
        for (int i = k + 1; i <= n; i++) {
            double l = P[(size_t)i * (n + 1) + k];
            if (l == 0)
                continue;
            l /= d;
            P[(size_t)i * (n + 1) + k] = l;
            for (int j = k + 1; j <= n; j++)
                P[(size_t)i * (n + 1) + j] -= l * P[(size_t)k * (n + 1) + j];
        }
    }
    memcpy(L, P, sizeof(double) * (size_t)(n + 1) * (n + 1));
    free(P);
    c->haveLU = 1;
    return 0;
}

static void sp_solve(port_t *c, double *b)
{
    port_plan_t *P = &c->plan;
    int n = c->n;
    double *w = c->work, *lux = c->lux;
    for (int k = 0; k < n; k++)
        w[k] = b[P->prow[k]];
    for (int l = 0; l < P->nflevels; l++)
        for (int r = P->fl_ptr[l]; r < P->fl_ptr[l + 1]; r++) {
            int k = P->fl_row[r];
            double acc = w[k];
            for (int q = P->lr_ptr[k]; q < P->lr_ptr[k + 1]; q++)
                acc -= lux[P->lr_pos[q]] * w[P->lr_col[q]];
            w[k] = acc;
        }
    for (int l = 0; l < P->nblevels; l++)
        for (int r = P->bl_ptr[l]; r < P->bl_ptr[l + 1]; r++) {
            int k = P->bl_row[r];
            double acc = w[k];
            for (int q = P->ur_ptr[k]; q < P->ur_ptr[k + 1]; q++)
                acc -= lux[P->ur_pos[q]] * w[P->ur_col[q]];
            w[k] = acc / lux[P->cdiag[k]];
        }
    for (int k = 0; k < n; k++)
        b[P->pcol[k]] = w[k];
}

static void lu_solve(port_t *c, double *b)
{
    int n = c->n;
    if (c->sparse) {
        sp_solve(c, b);
        return;
    }
    double *L = c->LU;
    double *y = malloc(sizeof(double) * (n + 1));
    for (int i = 1; i <= n; i++) {
        double acc = b[c->perm[i]];
        for (int k = 1; k < i; k++)
            acc -= L[(size_t)i * (n + 1) + k] * y[k];
        y[i] = acc;
    }
    for (int i = n; i >= 1; i--) {
        double acc = y[i];
        for (int k = i + 1; k <= n; k++)
            acc -= L[(size_t)i * (n + 1) + k] * y[k];
        y[i] = acc / L[(size_t)i * (n + 1) + i];
    }
    for (int i = 1; i <= n; i++)
        b[i] = y[i];
    free(y);
}

/* ------------------------------------------------------------------ */
static int conv_test(port_t *c)
{
    for (int i = 1; i <= c->n; i++) {
        double nw = c->rhs[i], od = c->rhsOld[i];
        if (isnan(nw))
            return 1;
        double tol = c->reltol * MAX(fabs(od), fabs(nw)) + (c->ntype[i] ? c->vntol : c->abstol);
        if (fabs(nw - od) > tol)
            return 1;
    }
    /* CKTconvTest runs the device current tests, but returns their error
     * code (OK), and NIiter overwrites the CKTnoncon they set with this
     * function's return value: the device tests never change the result
     * (niconv.c:82-86, cktop.c:126-145, niiter.c:286-289). */
    (void)mos1_conv(c);
    return 0;
}

static void dump(port_t *c)
{
    if (c->ndump >= c->dumpcap || c->sparse)
        return;
    int n = c->n, k = c->ndump++;
    if (c->dump_ax)
        for (int r = 0; r <= n; r++)
            for (int j = 0; j <= n; j++)
                c->dump_ax[(size_t)k * (n + 1) * (n + 1) + (size_t)r * (n + 1) + j] = A_(c, r, j);
    if (c->dump_rhs)
        memcpy(c->dump_rhs + (size_t)k * (n + 1), c->rhs, sizeof(double) * (n + 1));
    if (c->dump_rhsold)
        memcpy(c->dump_rhsold + (size_t)k * (n + 1), c->rhsOld, sizeof(double) * (n + 1));
    if (c->dump_meta) {
        c->dump_meta[4 * k] = c->time;
        c->dump_meta[4 * k + 1] = c->delta;
        c->dump_meta[4 * k + 2] = c->mode;
        c->dump_meta[4 * k + 3] = c->order;
    }
}

static int ni_iter(port_t *c, int maxIter)
{
    int iterno = 0;
    if (maxIter < 100)
        maxIter = 100;
    for (;;) {
        int noncon = ckt_load(c);
        iterno++;
        dump(c);
        int repivot = (c->mode & MODEINITJCT) || ((c->mode & MODEINITTRAN) && iterno == 1) ||
                      c->shouldReorder;
        if (repivot) {
            c->shouldReorder = 0;
            c->reorders++;
        }
        int e = lu_factor(c, repivot);
        if (e && !repivot) {
            c->reorders++;
            e = lu_factor(c, 1);
        }
        if (e) {
            c->numIter += iterno;
            return e;
        }
        lu_solve(c, c->rhs);
        c->rhs[0] = 0;
        c->rhsOld[0] = 0;
        if (iterno > maxIter) {
            c->numIter += iterno;
            return E_ITERLIM;
        }
        if (noncon == 0 && iterno != 1)
            noncon = conv_test(c);
        else
            noncon = 1;
        if (c->mode & MODEINITFLOAT) {
            if (noncon == 0) {
                c->numIter += iterno;
                return 0;
            }
        } else if (c->mode & MODEINITJCT) {
            c->mode = (c->mode & ~INITF) | MODEINITFIX;
            c->shouldReorder = 1;
        } else if (c->mode & MODEINITFIX) {
            if (noncon == 0)
                c->mode = (c->mode & ~INITF) | MODEINITFLOAT;
        } else if (c->mode & MODEINITTRAN) {
            if (iterno <= 1)
                c->shouldReorder = 1;
            c->mode = (c->mode & ~INITF) | MODEINITFLOAT;
        } else if (c->mode & MODEINITPRED) {
            c->mode = (c->mode & ~INITF) | MODEINITFLOAT;
        }
        double *t = c->rhs;
        c->rhs = c->rhsOld;
        c->rhsOld = t;
    }
}

/* ------------------------------------------------------------------ */
/* CKTop with dynamic_gmin, new_gmin and gillespie_src                  */
/* ------------------------------------------------------------------ */
static void op_zero(port_t *c)
{
    memset(c->rhsOld, 0, sizeof(double) * (c->n + 1));
    memset(c->states[0], 0, sizeof(double) * c->nstates);
}
static void op_save(port_t *c)
{
    memcpy(c->opsave_rhs, c->rhsOld, sizeof(double) * (c->n + 1));
    memcpy(c->opsave_st, c->states[0], sizeof(double) * c->nstates);
}
static void op_restore(port_t *c)
{
    memcpy(c->rhsOld, c->opsave_rhs, sizeof(double) * (c->n + 1));
    memcpy(c->states[0], c->opsave_st, sizeof(double) * c->nstates);
}

static int gmin_stepping(port_t *c, int trueGmin, int firstmode, int contmode)
{
    const int itl2 = 50;
    double factor = 10, oldGmin = 1e-2, gtarget, startgmin = c->gmin;
    int converged;
    c->mode = firstmode;
    op_zero(c);
    if (trueGmin) {
        c->gmin = oldGmin / factor;
        gtarget = MAX(startgmin, 0.0);
    } else {
        c->diagGmin = oldGmin / factor;
        gtarget = MAX(c->gmin, 0.0);
    }
    for (;;) {
        long before = c->numIter;
        converged = ni_iter(c, itl2);
        long iters = c->numIter - before;
        double g = trueGmin ? c->gmin : c->diagGmin;
        if (converged == 0) {
            c->mode = contmode;
            if (g <= gtarget)
                break;
            op_save(c);
            if (iters <= (itl2 / 4)) {
                factor *= sqrt(factor);
                if (factor > 10)
                    factor = 10;
            }
            if (iters > (3 * itl2 / 4))
                factor = trueGmin ? MAX(sqrt(factor), 3) : MAX(sqrt(factor), 1.00005);
            oldGmin = g;
            if (g < factor * gtarget) {
                factor = g / gtarget;
                g = gtarget;
            } else {
                g /= factor;
            }
        } else {
            if (factor < 1.00005)
                break;
            factor = sqrt(sqrt(factor));
            g = oldGmin / factor;
            op_restore(c);
        }
        if (trueGmin)
            c->gmin = g;
        else
            c->diagGmin = g;
    }
    if (trueGmin)
        c->gmin = MAX(startgmin, 0.0);
    else
        c->diagGmin = 0;
    return ni_iter(c, c->itl1);
}

static int gillespie_src(port_t *c, int firstmode, int contmode)
{
    const int itl2 = 50;
    double gminstart = c->gmin, convFact = 0, raise = 0.001;
    int converged;
    c->mode = firstmode;
    c->srcFact = 0;
    op_zero(c);
    converged = ni_iter(c, itl2);
    if (converged != 0) {
        c->diagGmin = c->gmin;
        for (int i = 0; i < 10; i++)
            c->diagGmin *= 10;
        for (int i = 0; i <= 10; i++) {
            converged = ni_iter(c, itl2);
            if (converged != 0) {
                c->diagGmin = 0;
                break;
            }
            c->diagGmin /= 10;
            c->mode = contmode;
        }
        c->diagGmin = 0;
    }
    if (converged == 0) {
        op_save(c);
        c->srcFact = convFact + raise;
        do {
            long before = c->numIter;
            converged = ni_iter(c, itl2);
            long iters = c->numIter - before;
            c->mode = contmode;
            if (converged == 0) {
                convFact = c->srcFact;
                op_save(c);
                c->srcFact = convFact + raise;
                if (iters <= (itl2 / 4))
                    raise *= 1.5;
                if (iters > (3 * itl2 / 4))
                    raise *= 0.5;
            } else {
                if (c->srcFact - convFact < 1e-8)
                    break;
                raise /= 10;
                if (raise > 0.01)
                    raise = 0.01;
                c->srcFact = convFact;
                op_restore(c);
            }
            if (c->srcFact > 1)
                c->srcFact = 1;
        } while ((raise >= 1e-7) && (convFact < 1));
        c->diagGmin = c->gmin = gminstart;
    }
    c->srcFact = 1;
    return convFact != 1 ? E_ITERLIM : 0;
}

static int op_solve(port_t *c)
{
    const int firstmode = MODETRANOP | MODEINITJCT, contmode = MODETRANOP | MODEINITFLOAT;
    c->mode = firstmode;
    if (ni_iter(c, c->itl1) == 0)
        return 0;
    if (gmin_stepping(c, 0, firstmode, contmode) == 0)
        return 0;
    if (gmin_stepping(c, 1, firstmode, contmode) == 0)
        return 0;
    return gillespie_src(c, firstmode, contmode);
}

/* ------------------------------------------------------------------ */
static int set_break(port_t *c, double time)
{
    double *b = c->breaks;
    if (almost_equal_ulps(time, c->time, 3))
        return 0;
    if (c->time > time)
        return 120;
    for (int i = 0; i < c->nbreaks; i++) {
        if (b[i] > time) {
            if ((b[i] - time) <= c->minbreak) {
                b[i] = time;
                return 0;
            }
            if (i > 0 && time - b[i - 1] <= c->minbreak)
                return 0;
            if (c->nbreaks >= c->breakcap) {
                c->breakcap *= 2;
                c->breaks = b = realloc(b, sizeof(double) * c->breakcap);
            }
            memmove(b + i + 1, b + i, sizeof(double) * (c->nbreaks - i));
            b[i] = time;
            c->nbreaks++;
            return 0;
        }
    }
    if (time - b[c->nbreaks - 1] <= c->minbreak)
        return 0;
    if (c->nbreaks >= c->breakcap) {
        c->breakcap *= 2;
        c->breaks = b = realloc(b, sizeof(double) * c->breakcap);
    }
    b[c->nbreaks++] = time;
    return 0;
}

static void clr_break(port_t *c)
{
    if (c->nbreaks > 2) {
        memmove(c->breaks, c->breaks + 1, sizeof(double) * (c->nbreaks - 1));
        c->nbreaks--;
    } else {
        c->breaks[0] = c->breaks[1];
        c->breaks[1] = c->tstop;
    }
}

static int src_accept_list(port_t *c, src_t *list, int cnt)
{
    for (int i = 0; i < cnt; i++) {
        src_t *h = &list[i];
        const double *cf = h->coef;
        int nc = h->ncoef;
        if (h->kind == 1) {
            double TD = nc > 2 ? cf[2] : 0.0;
            double TR = nc > 3 && cf[3] > 0.0 ? cf[3] : c->tstep;
            double TF = nc > 4 && cf[4] > 0.0 ? cf[4] : c->tstep;
            double PW = nc > 5 && cf[5] >= 0.0 ? cf[5] : 0.0;
            double PER = nc > 6 && cf[6] > 0.0 ? cf[6] : TR + TF + PW;
            double PHASE = nc > 7 ? cf[7] : 0.0;
            double time = c->time - TD;
            if (PHASE > 0.0 && time > PHASE * PER)
                continue;
            if (c->time >= h->brk) {
                double wait;
                if (time >= PER)
                    time -= PER * floor(time / PER);
                double atime = time + c->minbreak;
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
                h->brk = c->time + wait;
                int e = set_break(c, h->brk);
                if (e)
                    return e;
                h->brk -= c->minbreak;
            }
        } else if (h->kind == 4) {
            if (c->time >= h->brk) {
                double time = c->time;
                if (time > cf[nc - 2]) {
                    h->brk = c->tstop;
                    continue;
                }
                double atime = time + c->minbreak;
                for (int k = 0; k < nc; k += 2) {
                    if (cf[k] > atime) {
                        h->brk = c->time + cf[k] - time;
                        int e = set_break(c, h->brk);
                        if (e)
                            return e;
                        h->brk -= c->minbreak;
                        break;
                    }
                }
            }
        }
    }
    return 0;
}

static double terr(port_t *c, int qcap, double timeStep)
{
    double *s0 = c->states[0], *s1 = c->states[1];
    int ccap = qcap + 1;
    double volttol = c->abstol + c->reltol * MAX(fabs(s0[ccap]), fabs(s1[ccap]));
    double chargetol = MAX(fabs(s0[qcap]), fabs(s1[qcap]));
    chargetol = c->reltol * MAX(chargetol, c->chgtol) / c->delta;
    double tol = MAX(volttol, chargetol);
    double diff[8], deltmp[8];
    int i, j;
    for (i = c->order + 1; i >= 0; i--)
        diff[i] = c->states[i][qcap];
    for (i = 0; i <= c->order; i++)
        deltmp[i] = c->deltaOld[i];
    j = c->order;
    for (;;) {
        for (i = 0; i <= j; i++)
            diff[i] = (diff[i] - diff[i + 1]) / deltmp[i];
        if (--j < 0)
            break;
        for (i = 0; i <= j; i++)
            deltmp[i] = deltmp[i + 1] + c->deltaOld[i];
    }
    static const double trapCoeff[] = {.5, .08333333333};
    static const double gearCoeff[] = {.5, .2222222222};
    double factor = c->method == 1 ? gearCoeff[c->order - 1] : trapCoeff[c->order - 1];
    double del = c->trtol * tol / MAX(c->abstol, factor * fabs(diff[0]));
    if (c->order == 2)
        del = sqrt(del);
    return MIN(timeStep, del);
}

static double trunc_step(port_t *c, double timeStep)
{
    double t = 1e300;
    for (int i = 0; i < c->nb4; i++) {
        t = terr(c, c->b4[i].st + 11, t);   /* qb */
        t = terr(c, c->b4[i].st + 13, t);   /* qg */
        t = terr(c, c->b4[i].st + 15, t);   /* qd */
    }
    for (int i = 0; i < c->ncap; i++)
        t = terr(c, c->cap[i].st, t);
    for (int i = 0; i < c->ndio; i++)
        t = terr(c, c->dio[i].st + 6, t);   /* capCharge */
    for (int i = 0; i < c->nmos1; i++) {
        t = terr(c, c->mos1[i].st + S_QGS, t);
        t = terr(c, c->mos1[i].st + S_QGD, t);
        t = terr(c, c->mos1[i].st + S_QGB, t);
    }
    return MIN(2 * timeStep, t);
}

/* Gear coefficients, orders 1-2 (nicomcof.c:52-130): the corrector
 * system's row j holds the j-th powers of the summed past steps over
 * delta; right-hand side (0, -1/delta, 0); first column (1, 0, 0) */
static void comcof_gear(port_t *c)
{
    const int q = c->order;
    double m[3][3];
    int i, j, k;
    memset(c->ag, 0, sizeof c->ag);
    c->ag[1] = -1 / c->delta;
    double sum = 0;
    for (i = 0; i <= q; i++)
        m[0][i] = 1;
    for (i = 1; i <= q; i++)
        m[i][0] = 0;
    for (i = 1; i <= q; i++) {
        sum += c->deltaOld[i - 1];
        double pw = 1;
        for (j = 1; j <= q; j++) {
            pw *= sum / c->delta;
            m[j][i] = pw;
        }
    }
    for (i = 1; i <= q; i++)
        for (j = i + 1; j <= q; j++) {
            m[j][i] /= m[i][i];
            for (k = i + 1; k <= q; k++)
                m[j][k] -= m[j][i] * m[i][k];
        }
    for (i = 1; i <= q; i++)
        for (j = i + 1; j <= q; j++)
            c->ag[j] = c->ag[j] - m[j][i] * c->ag[i];
    c->ag[q] /= m[q][q];
    for (i = q - 1; i >= 0; i--) {
        for (j = i + 1; j <= q; j++)
            c->ag[i] = c->ag[i] - m[i][j] * c->ag[j];
        c->ag[i] /= m[i][i];
    }
}

static void comcof(port_t *c)
{
    if (c->method == 1) {
        comcof_gear(c);
        return;
    }
    if (c->order == 1) {
        c->ag[0] = 1 / c->delta;
        c->ag[1] = -1 / c->delta;
    } else {
        c->ag[0] = 1.0 / c->delta / (1.0 - c->xmu);
        c->ag[1] = c->xmu / (1.0 - c->xmu);
    }
}

/* stats: numIter, tranIter, timePts, accepted, rejected, status, opIter, npoints */
int port_run(port_t *c, long *stats, long maxSteps)
{
    int status = 0, firsttime = 1, maxOrder = c->maxord;
    double delta, olddelta, newdelta;
    long steps = 0;
    c->breakcap = 64;
    c->breaks = realloc(c->breaks, sizeof(double) * c->breakcap);
    for (int i = 0; i < c->nvsrc; i++)
        c->vsrc[i].brk = -1.0;
    for (int i = 0; i < c->nisrc; i++)
        c->isrc[i].brk = -1.0;
    c->gmin = c->gmin0;
    c->diagGmin = 0;
    c->srcFact = 1;
    delta = MIN(c->tstop / 100, c->tstep) / 10;
    c->breaks[0] = 0;
    c->breaks[1] = c->tstop;
    c->nbreaks = 2;
    c->time = 0;
    c->delta = 0;
    c->order = 1;
    if (op_solve(c) != 0) {
        status = E_NOOP;
        goto done;
    }
    c->opIter = c->numIter;
    c->timePts++;
    c->order = 1;
    for (int i = 0; i < 7; i++)
        c->deltaOld[i] = c->tmax;
    c->delta = delta;
    c->saveDelta = c->tstop / 50;
    c->mode = MODETRAN | MODEINITTRAN;
    c->ag[0] = c->ag[1] = 0;
    memcpy(c->states[1], c->states[0], sizeof(double) * c->nstates);
    for (;;) {
        /* nextTime */
        int e = src_accept_list(c, c->vsrc, c->nvsrc);
        if (!e)
            e = src_accept_list(c, c->isrc, c->nisrc);
        if (e) {
            status = e;
            goto done;
        }
        if (c->time > c->breaks[0])
            clr_break(c);
        c->accepted++;
        if (c->time >= c->tstart && c->out && c->npoints < c->outcap) {
            double *row = c->out + (size_t)c->npoints * (c->n + 1);
            row[0] = c->time;
            memcpy(row + 1, c->rhsOld + 1, sizeof(double) * c->n);
        }
        if (c->time >= c->tstart)
            c->npoints++;
        if (almost_equal_ulps(c->time, c->tstop, 100))
            goto done;
        if (++steps > maxSteps) {
            status = 121;
            goto done;
        }
        /* resume */
        c->delta = MIN(c->delta, c->tmax);
        if (almost_equal_ulps(c->time, c->breaks[0], 100) || c->breaks[0] - c->time <= c->delmin) {
            c->order = 1;
            c->delta = MIN(c->delta, .1 * MIN(c->saveDelta, c->breaks[1] - c->breaks[0]));
            if (firsttime)
                c->delta /= 10;
        }
        while ((c->breaks[0] <= c->time + c->minbreak ||
                almost_equal_ulps(c->breaks[0], c->time, 100)) && c->breaks[0] < c->tstop)
            clr_break(c);
        if (c->time + c->delta > c->breaks[0]) {
            c->saveDelta = c->delta;
            c->delta = c->breaks[0] - c->time;
        } else if (c->time + 1.9 * c->delta > c->breaks[0]) {
            c->saveDelta = c->delta;
            c->delta = (c->breaks[0] - c->time) / 2.;
        }
        for (int i = 5; i >= 0; i--)
            c->deltaOld[i + 1] = c->deltaOld[i];
        c->deltaOld[0] = c->delta;
        {
            double *temp = c->states[maxOrder + 1];
            for (int i = maxOrder; i >= 0; i--)
                c->states[i + 1] = c->states[i];
            c->states[0] = temp;
        }
        for (;;) {
            olddelta = c->delta;
            c->time += c->delta;
            c->deltaOld[0] = c->delta;
            comcof(c);
            long before = c->numIter;
            int converged = ni_iter(c, c->itl4);
            c->tranIter += c->numIter - before;
            c->timePts++;
            c->mode = MODETRAN | MODEINITPRED;
            if (firsttime) {
                memcpy(c->states[2], c->states[1], sizeof(double) * c->nstates);
                memcpy(c->states[3], c->states[1], sizeof(double) * c->nstates);
            }
            if (converged == E_SINGULAR) {
                status = converged;
                goto done;
            }
            if (converged != 0) {
                c->time = c->time - c->delta;
                c->rejected++;
                c->delta = c->delta / 8;
                if (firsttime)
                    c->mode = MODETRAN | MODEINITTRAN;
                c->order = 1;
                /* the engine's rule: the retry after a Newton failure
                 * factors with pivots chosen on its own matrix */
                c->shouldReorder = 1;
            } else {
                if (firsttime) {
                    firsttime = 0;
                    break;
                }
                newdelta = trunc_step(c, c->delta);
                if (newdelta > .9 * c->delta) {
                    if (c->order == 1 && maxOrder > 1) {
                        c->order = 2;
                        newdelta = trunc_step(c, c->delta);
                        if (newdelta <= 1.05 * c->delta)
                            c->order = 1;
                    }
                    c->delta = newdelta;
                    break;
                }
                c->time = c->time - c->delta;
                c->rejected++;
                c->delta = newdelta;
            }
            if (c->delta <= c->delmin) {
                if (olddelta > c->delmin) {
                    c->delta = c->delmin;
                } else {
                    status = E_TIMESTEP;
                    goto done;
                }
            }
            if (++steps > maxSteps) {
                status = 121;
                goto done;
            }
        }
    }
done:
    stats[0] = c->numIter;
    stats[1] = c->tranIter;
    stats[2] = c->timePts;
    stats[3] = c->accepted;
    stats[4] = c->rejected;
    stats[5] = status;
    stats[6] = c->opIter;
    stats[7] = c->npoints;
    stats[8] = c->reorders;
    stats[9] = c->ndump;
    /* the last pivot plan of the sparse path: L+U entries, column levels,
     * right-looking levels, KLU-order blocks, multiply-adds */
    stats[10] = c->havePlan ? c->plan.nlu : 0;
    stats[11] = c->havePlan ? c->plan.nlevels : 0;
    stats[12] = c->havePlan ? c->plan.nrl_levels : 0;
    stats[13] = c->havePlan ? c->plan.btf_blocks : 0;
    stats[14] = c->havePlan ? (long)c->plan.flops : 0;
    return status;
}
