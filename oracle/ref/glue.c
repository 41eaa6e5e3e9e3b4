/*
 * Test infrastructure: glue that lets the reference ngspice transient path
 * (compiled unmodified from the reference source tree) run without its
 * interactive front end.  Only the test suite and the golden-fixture
 * generator use the binary built from this file; nothing in the product
 * links it.
 *
 * What lives here, and which reference part each item stands in for:
 *   - the device table, reduced to the seven device types of the transient
 *     path, in the same relative order as `static_devices[]`
 *     (src/spicelib/devices/dev.c:142-200), so CKTload visits device types in
 *     the reference order;
 *   - SIMinit (src/main.c:500-525) and the globals main.c / sharedspice.c
 *     define (SPfrontEnd, DEVmaxnum, physical constants);
 *   - a recording IFfrontEnd (OUTpBeginPlot / OUTpData) that captures every
 *     accepted time point that CKTdump (src/spicelib/analysis/cktdump.c:33)
 *     emits;
 *   - IFnewUid / IFdelUid over an INPtables symbol table, restating
 *     src/spicelib/parser/ifnewuid.c without the front-end `struct circ`;
 *   - stand-ins for front-end queries (cp_getvar, ft_find_analysis, ...)
 *     that return the batch-mode defaults.
 */
#include "ngspice/ngspice.h"
#include "ngspice/cktdefs.h"
#include "ngspice/devdefs.h"
#include "ngspice/ifsim.h"
#include "ngspice/inpdefs.h"
#include "ngspice/iferrmsg.h"
#include "ngspice/ftedefs.h"
#include "ngspice/compatmode.h"
#include "ngspice/mif.h"
#include "ngspice/const.h"
#include <stdarg.h>
#include <sys/time.h>
#include "ngspice/cpdefs.h"

#include "oracle_ref.h"

extern SPICEdev *get_bsim4_info(void);
extern SPICEdev *get_bsim4v7_info(void);
extern SPICEdev *get_cap_info(void);
extern SPICEdev *get_dio_info(void);
extern SPICEdev *get_isrc_info(void);
extern SPICEdev *get_mos1_info(void);
extern SPICEdev *get_res_info(void);
extern SPICEdev *get_vsrc_info(void);

extern IFsimulator SIMinfo;
extern int spice_num_analysis(void);
extern SPICEanalysis **spice_analysis_ptr(void);

/* Same relative order as the reference table: bsim4 < bsim4v7 < cap < dio <
 * isrc < mos1 < res < vsrc. */
static SPICEdev *(*oracle_devices[])(void) = {
    get_bsim4_info, get_bsim4v7_info, get_cap_info, get_dio_info, get_isrc_info,
    get_mos1_info, get_res_info, get_vsrc_info,
};
#define ORACLE_NDEV ((int)(sizeof(oracle_devices) / sizeof(oracle_devices[0])))

SPICEdev **DEVices = NULL;
int DEVmaxnum = 0;
int *DEVicesfl = NULL;
IFfrontEnd *SPfrontEnd = NULL;
IFsimulator *ft_sim = NULL;
char Spice_Version[] = "46";

double CONSTroot2 = CONSTsqrt2;
double CONSTvt0 = CONSTboltz * REFTEMP / CHARGE;
double CONSTKoverQ = CONSTboltz / CHARGE;
double CONSTe = CONSTnap;

bool ft_ngdebug = FALSE;
bool ft_stricterror = FALSE;
bool ft_noinitprint = TRUE;
bool ft_noacctprint = TRUE;
bool wantevtdata = FALSE;
char *errMsg = NULL;
char *errRtn = NULL;
struct compat newcompat;
struct dbcomm *dbs = NULL;
FILE *cp_err = NULL;
int fixme_inoise_type = 0;
int fixme_onoise_type = 0;
Mif_Info_t g_mif_info;

static struct circ oracle_circ;
struct circ *ft_curckt = &oracle_circ;

int DEVflag(int type) { (void)type; return 0; }
int num_devices(void) { return ORACLE_NDEV; }
IFdevice **devices_ptr(void) { return (IFdevice **)DEVices; }
SPICEdev **devices(void) { return DEVices; }

/* ---------------------------------------------------------------- */
/* front-end stand-ins                                               */
/* ---------------------------------------------------------------- */
/* Front-end variables all read as unset, except "num_threads" (the
 * `set num_threads=N` of the reference, read by CKTsetup under USE_OMP),
 * which comes from the ORACLE_NUM_THREADS environment variable. */
bool cp_getvar(char *name, enum cp_types type, void *retval, size_t rsize)
{
    (void)rsize;
    if (name && !strcmp(name, "num_threads") && type == CP_NUM && retval) {
        const char *e = getenv("ORACLE_NUM_THREADS");
        if (e && atoi(e) > 0) {
            *(int *)retval = atoi(e);
            return TRUE;
        }
    }
    return FALSE;
}

int ft_find_analysis(char *name)
{
    int j;
    for (j = 0; j < ft_sim->numAnalyses; j++)
        if (strcmp(ft_sim->analyses[j]->name, name) == 0)
            return j;
    return -1;
}

IFparm *ft_find_analysis_parm(int which, char *name)
{
    int i;
    for (i = 0; i < ft_sim->analyses[which]->numParms; i++)
        if (!strcmp(ft_sim->analyses[which]->analysisParms[i].keyword, name))
            return &(ft_sim->analyses[which]->analysisParms[i]);
    return NULL;
}

void controlled_exit(int status)
{
    fprintf(stderr, "oracle: controlled_exit(%d)\n", status);
    exit(status ? status : 1);
}

void inp_evaluate_temper(struct circ *c) { (void)c; }
bool check_autostop(char *what) { (void)what; return FALSE; }
bool ft_stepcheck(void) { return FALSE; }

int IFnewUid(CKTcircuit *ckt, IFuid *newuid, IFuid olduid, char *suffix,
             int type, CKTnode **nodedata)
{
    char *newname;
    int error;
    if (olduid)
        newname = tprintf("%s#%s", (char *)olduid, suffix);
    else
        newname = tprintf("%s", suffix);
    switch (type) {
    case UID_ANALYSIS:
    case UID_TASK:
    case UID_INSTANCE:
    case UID_OTHER:
    case UID_MODEL:
        error = INPinsert(&newname, ft_curckt->ci_symtab);
        if (error && error != E_EXISTS)
            return error;
        *newuid = newname;
        break;
    case UID_SIGNAL:
        error = INPmkTerm(ckt, &newname, ft_curckt->ci_symtab, nodedata);
        if (error && error != E_EXISTS)
            return error;
        *newuid = newname;
        break;
    default:
        return E_BADPARM;
    }
    return OK;
}

int IFdelUid(CKTcircuit *ckt, IFuid uid, int type)
{
    (void)ckt; (void)uid; (void)type;
    return OK;
}

static int fe_pause(void) { return 0; }

static double fe_seconds(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

static void fe_error(int flags, char *msg, IFuid *names)
{
    (void)names;
    if (flags & (ERR_FATAL | ERR_PANIC))
        fprintf(stderr, "oracle: error: %s\n", msg);
}

static void fe_errorf(int flags, const char *fmt, ...)
{
    va_list ap;
    if (!(flags & (ERR_FATAL | ERR_PANIC | ERR_WARNING)))
        return;
    va_start(ap, fmt);
    fprintf(stderr, "oracle: ");
    vfprintf(stderr, fmt, ap);
    va_end(ap);
}

/* ---------------------------------------------------------------- */
/* recording output: every accepted point CKTdump hands over          */
/* ---------------------------------------------------------------- */
oracle_trace_t oracle_trace;

static int fe_begin_plot(CKTcircuit *ckt, JOB *job, IFuid name, IFuid ref,
                         int reftype, int num, IFuid *names, int type,
                         runDesc **plot)
{
    int i;
    (void)ckt; (void)job; (void)name; (void)ref; (void)reftype; (void)type;
    if (num == 666 && names == NULL) {   /* rawfile relink on resume */
        *plot = (runDesc *)&oracle_trace;
        return OK;
    }
    oracle_trace.nvars = num;
    oracle_trace.names = TMALLOC(char *, num);
    for (i = 0; i < num; i++)
        oracle_trace.names[i] = copy((char *)names[i]);
    oracle_trace.npoints = 0;
    *plot = (runDesc *)&oracle_trace;
    return OK;
}

static int fe_data(runDesc *plot, IFvalue *ref, IFvalue *val)
{
    oracle_trace_t *t = (oracle_trace_t *)plot;
    int n = val->v.numValue;
    if (n > t->nvars)
        n = t->nvars;
    if (t->npoints == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 1024;
        t->times = TREALLOC(double, t->times, t->cap);
        t->values = TREALLOC(double, t->values, (size_t)t->cap * (size_t)t->nvars);
    }
    t->times[t->npoints] = ref->rValue;
    memcpy(t->values + (size_t)t->npoints * (size_t)t->nvars, val->v.vec.rVec,
           (size_t)n * sizeof(double));
    t->npoints++;
    return OK;
}

static int fe_end_plot(runDesc *plot) { (void)plot; return OK; }

static int fe_attributes(runDesc *plot, IFuid name, int param, IFvalue *val)
{
    (void)plot; (void)name; (void)param; (void)val;
    return OK;
}

static IFfrontEnd oracle_frontend = {
    IFnewUid, IFdelUid, fe_pause, fe_seconds, fe_error, fe_errorf,
    fe_begin_plot, fe_data, fe_end_plot, fe_attributes,
};

/* Restates SIMinit (src/main.c:500-525) for the reduced device table. */
void oracle_init(void)
{
    int i;
    DEVices = TMALLOC(SPICEdev *, ORACLE_NDEV);
    DEVicesfl = TMALLOC(int, ORACLE_NDEV);
    for (i = 0; i < ORACLE_NDEV; i++)
        DEVices[i] = oracle_devices[i]();
    SIMinfo.numDevices = DEVmaxnum = ORACLE_NDEV;
    SIMinfo.devices = devices_ptr();
    SIMinfo.numAnalyses = spice_num_analysis();
    SIMinfo.analyses = (IFanalysis **)spice_analysis_ptr();
    SPfrontEnd = &oracle_frontend;
    ft_sim = &SIMinfo;
    cp_err = stderr;
    memset(&g_mif_info, 0, sizeof(g_mif_info));
}
