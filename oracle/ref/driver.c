/*
 * Test infrastructure: batch driver for the reference ngspice transient path.
 *
 *   ngspice_ref NETLIST OUT.bin [--iters ITERS.bin] [--max-iters N]
 *               [--states STATES.bin] [--states-every K]
 *
 * Reads a flat netlist (no .subckt, no .param, no braces), hands its cards
 * to the reference parser passes INPpas1/INPpas2/INPpas4/INPpas3 in the order
 * if_inpdeck uses (src/frontend/spiceif.c:100-196), runs the deck's analyses
 * with CKTdoJob exactly as the front end's "run" command does
 * (src/frontend/spiceif.c:221, doAnalyses(ckt, 1, task)), and writes every
 * accepted time point plus the reference's run statistics to OUT.bin.
 *
 * With --iters, every Newton iteration's stamped matrix and right-hand side
 * (captured just before the reference factors them, through the linker
 * wrappers __wrap_SMPluFac / __wrap_SMPreorder) are written to ITERS.bin,
 * up to N iterations (default 2000).
 *
 * With --states STATES.bin [--states-every K], every K-th captured
 * iteration also records the linearisation point CKTload started from:
 * CKTstates[0..2] as they were before the load (__wrap_CKTload snapshots
 * them; the load itself writes state 0, and state 1 in MODEINITTRAN),
 * the integration coefficients, gmin, srcFact, and each BSIM4 instance's
 * BSIM4von (kept between iterations for the gate-voltage limiting), in
 * the model / instance list order CKTload visits: 4.8 instances, then
 * version 4.7 (BSIM4v7) ones.  Record layout:
 *   int32 iteration index (0-based, as in ITERS.bin), int32 nstates,
 *   int32 nvon, int32 0, double ag[2], deltaOld[2], gmin, srcFact,
 *   nstates x double state0, state1, state2, nvon x double von.
 *
 * Output layout (little-endian):
 *   "NGOR" int32 version=1
 *   int32 nvars, int32 npoints
 *   nvars x (int32 len, bytes name)
 *   npoints x double time
 *   npoints x nvars x double value
 *   int32 stats[8] = numIter, tranIter, timePts, accepted, rejected,
 *                    status (CKTdoJob return), 0, 0
 *   double times[6] = tranTime, loadTime, decompTime, solveTime,
 *                     reorderTime, tranTruncTime
 */
#include "ngspice/ngspice.h"
#include "ngspice/cktdefs.h"
#include "ngspice/devdefs.h"
#include "ngspice/ifsim.h"
#include "ngspice/inpdefs.h"
#include "ngspice/iferrmsg.h"
#include "ngspice/ftedefs.h"
#include "ngspice/smpdefs.h"
#include "ngspice/tskdefs.h"
#include <ctype.h>

#include "bsim4/bsim4def.h"
#include "oracle_ref.h"

extern IFsimulator *ft_sim;
extern int IFnewUid(CKTcircuit *, IFuid *, IFuid, char *, int, CKTnode **);

/* ---------------------------------------------------------------- */
/* per-Newton-iteration capture                                      */
/* ---------------------------------------------------------------- */
static FILE *iter_fp = NULL;
static long iter_count = 0;
static long iter_max = 2000;
static CKTcircuit *iter_ckt = NULL;

int __real_SMPluFac(SMPmatrix *, double, double);
int __real_SMPreorder(SMPmatrix *, double, double, double);
int __real_CKTload(CKTcircuit *);

/* linearisation point of the iteration being loaded (--states) */
static FILE *states_fp = NULL;
static long states_every = 1;
static double *pre_st[3];
static double *pre_von;
static int pre_nst, pre_nvon, pre_cap_st, pre_cap_von, pre_valid;

static void snapshot_states(CKTcircuit *ckt)
{
    int k, nv = 0;
    int type = INPtypelook("BSIM4");
    BSIM4model *model;
    BSIM4instance *here;
    pre_valid = 0;
    if (ckt->CKTnumStates > pre_cap_st) {
        for (k = 0; k < 3; k++)
            pre_st[k] = TREALLOC(double, pre_st[k], ckt->CKTnumStates);
        pre_cap_st = ckt->CKTnumStates;
    }
    pre_nst = ckt->CKTnumStates;
    for (k = 0; k < 3; k++)
        memcpy(pre_st[k], ckt->CKTstates[k], sizeof(double) * (size_t)pre_nst);
    if (type >= 0)
        for (model = (BSIM4model *)ckt->CKThead[type]; model; model = BSIM4nextModel(model))
            for (here = BSIM4instances(model); here; here = BSIM4nextInstance(here)) {
                if (nv >= pre_cap_von) {
                    pre_cap_von = 2 * pre_cap_von + 64;
                    pre_von = TREALLOC(double, pre_von, pre_cap_von);
                }
                pre_von[nv++] = here->BSIM4von;
            }
    /* then the version 4.7 instances: BSIM4v7 follows BSIM4 in the device
     * table, so CKTload reaches them after every 4.8 instance */
    nv = oracle_v47_von(ckt, &pre_von, &pre_cap_von, nv);
    pre_nvon = nv;
    pre_valid = 1;
}

int __wrap_CKTload(CKTcircuit *ckt)
{
    if (states_fp && ckt == iter_ckt && iter_count < iter_max &&
        iter_count % states_every == 0)
        snapshot_states(ckt);
    else
        pre_valid = 0;
    return __real_CKTload(ckt);
}

static void dump_states(CKTcircuit *ckt, long index)
{
    int32_t hdr[4];
    double d[6];
    if (!states_fp || !pre_valid)
        return;
    pre_valid = 0;
    hdr[0] = (int32_t)index;
    hdr[1] = pre_nst;
    hdr[2] = pre_nvon;
    hdr[3] = 0;
    fwrite(hdr, sizeof(int32_t), 4, states_fp);
    d[0] = ckt->CKTag[0];
    d[1] = ckt->CKTag[1];
    d[2] = ckt->CKTdeltaOld[0];
    d[3] = ckt->CKTdeltaOld[1];
    d[4] = ckt->CKTgmin;
    d[5] = ckt->CKTsrcFact;
    fwrite(d, sizeof(double), 6, states_fp);
    fwrite(pre_st[0], sizeof(double), (size_t)pre_nst, states_fp);
    fwrite(pre_st[1], sizeof(double), (size_t)pre_nst, states_fp);
    fwrite(pre_st[2], sizeof(double), (size_t)pre_nst, states_fp);
    fwrite(pre_von, sizeof(double), (size_t)pre_nvon, states_fp);
}

/* Writes one record: time, delta, mode, order, n, nnz, then nnz x
 * (int32 row, int32 col, double value) in external 1-based equation
 * numbers, then rhs[0..n].  The matrix is read in the CSC form KLU
 * holds after CKTload (klusmp.c:137-323 builds it; Ax columns are in the
 * collapsed numbering mapped back through NodeCollapsingNewToOld). */
static void dump_iteration(SMPmatrix *m, const char *kind)
{
    CKTcircuit *ckt = iter_ckt;
    KLUmatrix *k;
    int n, j, p, nnz;
    int32_t hdr[4];
    double dh[2];
    if (!iter_fp || !ckt || iter_count >= iter_max)
        return;
    k = m->SMPkluMatrix;
    if (!m->CKTkluMODE || !k || !k->KLUmatrixAx)
        return;
    iter_count++;
    n = (int)k->KLUmatrixN;
    nnz = (int)k->KLUmatrixNZ;
    fwrite(kind, 1, 4, iter_fp);
    dh[0] = ckt->CKTtime;
    dh[1] = ckt->CKTdelta;
    fwrite(dh, sizeof(double), 2, iter_fp);
    hdr[0] = (int32_t)ckt->CKTmode;
    hdr[1] = ckt->CKTorder;
    hdr[2] = (int32_t)k->KLUmatrixNrhs;
    hdr[3] = nnz;
    fwrite(hdr, sizeof(int32_t), 4, iter_fp);
    for (j = 0; j < n; j++) {
        for (p = k->KLUmatrixAp[j]; p < k->KLUmatrixAp[j + 1]; p++) {
            int32_t rc[2];
            int r = k->KLUmatrixAi[p];
            if (k->KLUmatrixNodeCollapsingNewToOld) {
                rc[0] = (int32_t)k->KLUmatrixNodeCollapsingNewToOld[r];
                rc[1] = (int32_t)k->KLUmatrixNodeCollapsingNewToOld[j];
            } else {
                rc[0] = r + 1;
                rc[1] = j + 1;
            }
            fwrite(rc, sizeof(int32_t), 2, iter_fp);
            fwrite(&k->KLUmatrixAx[p], sizeof(double), 1, iter_fp);
        }
    }
    fwrite(ckt->CKTrhs, sizeof(double), (size_t)k->KLUmatrixNrhs + 1, iter_fp);
    fwrite(ckt->CKTrhsOld, sizeof(double), (size_t)k->KLUmatrixNrhs + 1, iter_fp);
    dump_states(ckt, iter_count - 1);
}

int __wrap_SMPluFac(SMPmatrix *m, double pivtol, double gmin)
{
    dump_iteration(m, "LUFC");
    return __real_SMPluFac(m, pivtol, gmin);
}

int __wrap_SMPreorder(SMPmatrix *m, double pivtol, double pivrel, double gmin)
{
    dump_iteration(m, "REOR");
    return __real_SMPreorder(m, pivtol, pivrel, gmin);
}

/* ---------------------------------------------------------------- */
/* netlist reading                                                   */
/* ---------------------------------------------------------------- */
static struct card *new_card(char *line, int num)
{
    struct card *c = TMALLOC(struct card, 1);
    c->linenum = num;
    c->linenum_orig = num;
    c->line = line;
    return c;
}

/* Flat-netlist reader: lower-cases, joins '+' continuation lines, drops
 * comment lines and the output/control cards the transient path ignores. */
static struct card *read_deck(const char *path, int *ncards)
{
    FILE *fp = fopen(path, "r");
    char buf[65536];
    struct card *head = NULL, *tail = NULL;
    int num = 0, incontrol = 0;
    if (!fp) {
        fprintf(stderr, "oracle: cannot open %s\n", path);
        exit(2);
    }
    while (fgets(buf, sizeof buf, fp)) {
        char *s = buf, *e;
        size_t len = strlen(buf);
        while (len && (buf[len - 1] == '\n' || buf[len - 1] == '\r'))
            buf[--len] = '\0';
        for (e = buf; *e; e++)
            *e = (char)tolower((unsigned char)*e);
        num++;
        if (num == 1) {                 /* title card */
            head = tail = new_card(copy(buf), num);
            continue;
        }
        while (*s == ' ' || *s == '\t')
            s++;
        if (*s == '\0' || *s == '*')
            continue;
        if (incontrol) {
            if (strncmp(s, ".endc", 5) == 0)
                incontrol = 0;
            continue;
        }
        if (strncmp(s, ".control", 8) == 0) {
            incontrol = 1;
            continue;
        }
        if ((e = strchr(s, ';')) != NULL)
            *e = '\0';
        if (*s == '+' && tail && tail != head) {
            char *joined = tprintf("%s %s", tail->line, s + 1);
            tfree(tail->line);
            tail->line = joined;
            continue;
        }
        if (strncmp(s, ".end", 4) == 0 && (s[4] == '\0' || isspace((unsigned char)s[4])))
            break;
        if (strncmp(s, ".print", 6) == 0 || strncmp(s, ".plot", 5) == 0 ||
            strncmp(s, ".save", 5) == 0 || strncmp(s, ".probe", 6) == 0 ||
            strncmp(s, ".width", 6) == 0 || strncmp(s, ".meas", 5) == 0)
            continue;
        tail->nextcard = new_card(copy(s), num);
        tail = tail->nextcard;
    }
    fclose(fp);
    *ncards = num;
    return head;
}

static void write_trace(const char *path, CKTcircuit *ckt, int status)
{
    FILE *fp = fopen(path, "wb");
    int32_t v;
    int i;
    int32_t st[8] = {0};
    double tm[6];
    oracle_trace_t *t = &oracle_trace;
    if (!fp) {
        fprintf(stderr, "oracle: cannot write %s\n", path);
        exit(2);
    }
    fwrite("NGOR", 1, 4, fp);
    v = 1;
    fwrite(&v, 4, 1, fp);
    v = t->nvars;
    fwrite(&v, 4, 1, fp);
    v = t->npoints;
    fwrite(&v, 4, 1, fp);
    for (i = 0; i < t->nvars; i++) {
        v = (int32_t)strlen(t->names[i]);
        fwrite(&v, 4, 1, fp);
        fwrite(t->names[i], 1, (size_t)v, fp);
    }
    fwrite(t->times, sizeof(double), (size_t)t->npoints, fp);
    fwrite(t->values, sizeof(double), (size_t)t->npoints * (size_t)t->nvars, fp);
    st[0] = ckt->CKTstat->STATnumIter;
    st[1] = ckt->CKTstat->STATtranIter;
    st[2] = ckt->CKTstat->STATtimePts;
    st[3] = ckt->CKTstat->STATaccepted;
    st[4] = ckt->CKTstat->STATrejected;
    st[5] = status;
    fwrite(st, 4, 8, fp);
    tm[0] = ckt->CKTstat->STATtranTime;
    tm[1] = ckt->CKTstat->STATloadTime;
    tm[2] = ckt->CKTstat->STATdecompTime;
    tm[3] = ckt->CKTstat->STATsolveTime;
    tm[4] = ckt->CKTstat->STATreorderTime;
    tm[5] = ckt->CKTstat->STATtranTruncTime;
    fwrite(tm, sizeof(double), 6, fp);
    fclose(fp);
}

int main(int argc, char **argv)
{
    struct card *deck, *c;
    int ncards, err, which, i, bad = 0;
    INPtables *tab;
    CKTcircuit *ckt;
    IFuid taskUid, optUid;
    TSKtask *task = NULL;
    JOB *opt = NULL;
    const char *iters_path = NULL;
    const char *states_path = NULL;

    if (argc < 3) {
        fprintf(stderr, "usage: %s NETLIST OUT.bin [--iters ITERS.bin] [--max-iters N]\n", argv[0]);
        return 2;
    }
    for (i = 3; i < argc; i++) {
        if (!strcmp(argv[i], "--iters") && i + 1 < argc)
            iters_path = argv[++i];
        else if (!strcmp(argv[i], "--max-iters") && i + 1 < argc)
            iter_max = atol(argv[++i]);
        else if (!strcmp(argv[i], "--states") && i + 1 < argc)
            states_path = argv[++i];
        else if (!strcmp(argv[i], "--states-every") && i + 1 < argc)
            states_every = atol(argv[++i]) > 0 ? atol(argv[i]) : 1;
    }

    oracle_init();
    deck = read_deck(argv[1], &ncards);
    tab = INPtabInit(ncards);
    ft_curckt->ci_symtab = tab;

    err = ft_sim->newCircuit(&ckt);
    if (err) { fprintf(stderr, "oracle: CKTinit failed %d\n", err); return 3; }
    ft_curckt->ci_ckt = ckt;
    err = IFnewUid(ckt, &taskUid, NULL, "default", UID_TASK, NULL);
    if (err) return 3;
    err = ft_sim->newTask(ckt, &task, taskUid, NULL);
    if (err) return 3;
    which = ft_find_analysis("options");
    if (which != -1) {
        err = IFnewUid(ckt, &optUid, NULL, "options", UID_ANALYSIS, NULL);
        if (err) return 3;
        err = ft_sim->newAnalysis(ckt, which, optUid, &opt, task);
        if (err) return 3;
    }
    ft_curckt->ci_defTask = task;
    ft_curckt->ci_curTask = task;

    INPpas1(ckt, deck->nextcard, tab);
    INPpas2(ckt, deck->nextcard, tab, task);
    INPpas4(ckt, tab);
    INPpas3(ckt, deck->nextcard, tab, task, ft_sim->nodeParms, ft_sim->numNodeParms);
    for (c = deck->nextcard; c; c = c->nextcard) {
        if (c->error) {
            fprintf(stderr, "oracle: card %d: %s\n  %s\n", c->linenum, c->line, c->error);
            if (!strstr(c->error, "arning") && !strstr(c->error, "ignored"))
                bad = 1;
        }
    }
    if (bad)
        return 4;

    if (iters_path) {
        iter_fp = fopen(iters_path, "wb");
        iter_ckt = ckt;
        if (states_path)
            states_fp = fopen(states_path, "wb");
    }
    err = ft_sim->doAnalyses(ckt, 1, task);
    if (getenv("ORACLE_KLU_STATS") && ckt->CKTmatrix && ckt->CKTmatrix->CKTkluMODE &&
        ckt->CKTmatrix->SMPkluMatrix) {
        /* fill and flops of KLU's last factorization (BTF + AMD ordering) */
        KLUmatrix *km = ckt->CKTmatrix->SMPkluMatrix;
        if (km->KLUmatrixSymbolic && km->KLUmatrixNumeric) {
            klu_flops(km->KLUmatrixSymbolic, km->KLUmatrixNumeric, km->KLUmatrixCommon);
            fprintf(stderr, "oracle: klu n=%d nnz=%d nblocks=%d maxblock=%d nzoff=%d lnz=%d unz=%d"
                    " flops=%.0f\n", (int)km->KLUmatrixN, (int)km->KLUmatrixNZ,
                    km->KLUmatrixSymbolic->nblocks, km->KLUmatrixSymbolic->maxblock,
                    km->KLUmatrixSymbolic->nzoff, km->KLUmatrixNumeric->lnz,
                    km->KLUmatrixNumeric->unz, km->KLUmatrixCommon->flops);
        }
    }
    if (iter_fp)
        fclose(iter_fp);
    if (states_fp)
        fclose(states_fp);
    if (err)
        fprintf(stderr, "oracle: doAnalyses returned %d\n", err);
    write_trace(argv[2], ckt, err);
    return err ? 5 : 0;
}
