/*
 * sharedspice-compatible C API of the GB300 transient engine.
 *
 * Every declaration below replaces the function or type of the same name
 * in the reference's shared-library interface,
 * src/include/ngspice/sharedspice.h (types :176-225, callbacks :247-319,
 * functions :384-515).  Struct layouts and prototypes are kept identical so
 * an application built against the reference header links against
 * libngspice_gb300.so unchanged.  Return codes follow the reference: 0 =
 * success, 1 = error (src/sharedspice.c:1124-1160).
 *
 * Scope: circuits and commands of the transient path (.tran on R/C/V/I,
 * diode, MOS1 and BSIM4 netlists).  Commands outside that path return 1
 * after reporting "unsupported command" through the SendChar callback.
 */
#ifndef NGSF_SHAREDSPICE_H
#define NGSF_SHAREDSPICE_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IMPEXP __attribute__((visibility("default")))

struct ngcomplex {
    double cx_real;
    double cx_imag;
};
typedef struct ngcomplex ngcomplex_t;

typedef bool NG_BOOL;

/* vector data owned by the library, valid until the next call */
typedef struct vector_info {
    char *v_name;
    int v_type;
    short v_flags;
    double *v_realdata;
    ngcomplex_t *v_compdata;
    int v_length;
} vector_info, *pvector_info;

typedef struct vecvalues {
    char *name;
    double creal;
    double cimag;
    NG_BOOL is_scale;
    NG_BOOL is_complex;
} vecvalues, *pvecvalues;

typedef struct vecvaluesall {
    int veccount;
    int vecindex;
    pvecvalues *vecsa;
} vecvaluesall, *pvecvaluesall;

typedef struct vecinfo {
    int number;
    char *vecname;
    NG_BOOL is_real;
    void *pdvec;
    void *pdvecscale;
} vecinfo, *pvecinfo;

typedef struct vecinfoall {
    char *name;
    char *title;
    char *date;
    char *type;
    int veccount;
    pvecinfo *vecs;
} vecinfoall, *pvecinfoall;

typedef int(SendChar)(char *, int, void *);
typedef int(SendStat)(char *, int, void *);
typedef int(ControlledExit)(int, NG_BOOL, NG_BOOL, int, void *);
typedef int(SendData)(pvecvaluesall, int, int, void *);
typedef int(SendInitData)(pvecinfoall, int, void *);
typedef int(BGThreadRunning)(NG_BOOL, int, void *);
typedef int(GetVSRCData)(double *, double, char *, int, void *);
typedef int(GetISRCData)(double *, double, char *, int, void *);
typedef int(GetSyncData)(double, double *, double, int, int, int, void *);

/* sharedspice.h:384 */
IMPEXP int ngSpice_Init(SendChar *printfcn, SendStat *statfcn, ControlledExit *ngexit,
                        SendData *sdata, SendInitData *sinitdata, BGThreadRunning *bgtrun,
                        void *userData);
/* sharedspice.h:398; with syncdat set, a transient stops at the two
 * points where the reference calls sharedsync (before each step, and after
 * each step's verdict) and calls syncdat there with the reference's
 * arguments and meaning (sharedspice.c:2437-2490): the callback may change
 * the next delta and, by returning 1, redo the step; delta is kept short of
 * the final time as the reference keeps it.  Each stop is a kernel exit and
 * relaunch.  The external-source callbacks (vsrcdat, isrcdat) are recorded
 * but not called: netlists with EXTERNAL sources are refused. */
IMPEXP int ngSpice_Init_Sync(GetVSRCData *vsrcdat, GetISRCData *isrcdat,
                             GetSyncData *syncdat, int *ident, void *userData);
/* sharedspice.h:403; a transient runs on the GPU in 64 windows of its
 * length: SendData fires once per accepted point, in order, as each window
 * ends; "bg_halt" stops a background run at the end of its current window
 * (state kept on the device) and "bg_resume" continues it. */
IMPEXP int ngSpice_Command(char *command);
/* sharedspice.h:407 */
IMPEXP pvector_info ngGet_Vec_Info(char *vecname);
/* sharedspice.h:465 */
IMPEXP int ngSpice_Circ(char **circarray);
/* sharedspice.h:470 */
IMPEXP char *ngSpice_CurPlot(void);
/* sharedspice.h:476 */
IMPEXP char **ngSpice_AllPlots(void);
/* sharedspice.h:482 */
IMPEXP char **ngSpice_AllVecs(char *plotname);
/* sharedspice.h:486 */
IMPEXP NG_BOOL ngSpice_running(void);
/* sharedspice.h:490; honoured for the next run (adds a breakpoint) */
IMPEXP NG_BOOL ngSpice_SetBkpt(double time);
/* sharedspice.h:494-515 */
IMPEXP int ngSpice_nospinit(void);
IMPEXP int ngSpice_nospiceinit(void);
IMPEXP int ngSpice_LockRealloc(void);
IMPEXP int ngSpice_UnlockRealloc(void);
IMPEXP int ngSpice_Reset(void);

#ifdef __cplusplus
}
#endif
#endif
