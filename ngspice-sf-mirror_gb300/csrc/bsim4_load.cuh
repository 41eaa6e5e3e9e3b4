/*
 * BSIM4 (level 54, version 4.8.3) device evaluation on the GPU: one thread
 * per instance, parameters in structure-of-arrays layout (csrc/bsim4.h),
 * stamps written to per-instance slots that the deterministic gather of
 * ckt_load sums in the reference's order.
 *
 * Follows BSIM4LoadOMP + BSIM4LoadRhsMat
 * (src/spicelib/devices/bsim4/b4ld.c:70-5623) for the default selectors
 * the compiler accepts: mobMod 0, capMod 2, rdsMod 0, rbodyMod 0,
 * rgateMod 0, trnqsMod 0, acnqsMod 0, igcMod 0, igbMod 0, dioMod 1,
 * tempMod 0, mtrlMod 0, gidlMod 0, cvchargeMod 0, no vtl/lambda
 * velocity terms, bypass off, NEWCONV defined, PREDICTOR undefined.
 * Anything else is rejected when the netlist is compiled.
 *
 * The arithmetic keeps the reference's operation order so that the stamped
 * Jacobian agrees to rounding with the reference build (which is compiled
 * without FMA contraction; this file is compiled with --fmad=false).
 */
#ifndef NGSF_BSIM4_LOAD_CUH
#define NGSF_BSIM4_LOAD_CUH

#include <math.h>
#include <stddef.h>

#include "bsim4.h"
#include "devsup.cuh"
#include "ngsf_types.h"

#define B4_MAX_EXP 5.834617425e14
#define B4_MIN_EXP 1.713908431e-15
#define B4_EXP_THRESHOLD 34.0
#define B4_EPSSI 1.03594e-10
#define B4_CHARGE_Q 1.60219e-19
#define B4_DELTA_1 0.02
#define B4_DELTA_3 0.02
#define B4_DELTA_4 0.02
/* elementary charge of the reference's const.h, used by the poly-depletion
 * helper (b4ld.c BSIM4polyDepletion uses CHARGE, not Charge_q) */
#define B4_CHARGE 1.6021766208e-19

/* bounded exponential with derivative (b4ld.c DEXP(A,B,C)) */
NGSF_HD inline void b4_dexp(double a, double &b, double &c)
{
    if (a > B4_EXP_THRESHOLD) {
        b = B4_MAX_EXP * (1.0 + a - B4_EXP_THRESHOLD);
        c = B4_MAX_EXP;
    } else if (a < -B4_EXP_THRESHOLD) {
        b = B4_MIN_EXP;
        c = 0;
    } else {
        b = exp(a);
        c = b;
    }
}

/* poly-gate depletion (b4ld.c BSIM4polyDepletion) */
NGSF_HD inline void b4_poly_depletion(double phi, double ngate, double epsgate,
                                                  double coxe, double Vgs, double &Vgs_eff,
                                                  double &dVgs_eff_dVg)
{
    if ((ngate > 1.0e18) && (ngate < 1.0e25) && (Vgs > phi) && (epsgate != 0)) {
        double T1 = 1.0e6 * B4_CHARGE * epsgate * ngate / (coxe * coxe);
        double T8 = Vgs - phi;
        double T4 = sqrt(1.0 + 2.0 * T8 / T1);
        double T2 = 2.0 * T8 / (T4 + 1.0);
        double T3 = 0.5 * T2 * T2 / T1;
        double T7 = 1.12 - T3 - 0.05;
        double T6 = sqrt(T7 * T7 + 0.224);
        double T5 = 1.12 - 0.5 * (T7 + T6);
        Vgs_eff = Vgs - T5;
        dVgs_eff_dVg = 1.0 - (0.5 - 0.5 / T4) * (1.0 + T7 / T6);
    } else {
        Vgs_eff = Vgs;
        dVgs_eff_dVg = 1.0;
    }
}

/* junction current of one side, dioMod 1 (b4ld.c:792-813 / 862-883) */
NGSF_HD inline void b4_junction_dio1(double SatCurrent, double Nvtm, double vjmFwd,
                                                 double IVjmFwd, double v, double gmin,
                                                 double &g, double &c)
{
    if (SatCurrent <= 0.0) {
        g = gmin;
        c = g * v;
        return;
    }
    double T2 = v / Nvtm;
    if (T2 < -B4_EXP_THRESHOLD) {
        g = gmin;
        c = SatCurrent * (B4_MIN_EXP - 1.0) + gmin * v;
    } else if (v <= vjmFwd) {
        double ev = exp(T2);
        g = SatCurrent * ev / Nvtm + gmin;
        c = SatCurrent * (ev - 1.0) + gmin * v;
    } else {
        double T0 = IVjmFwd / Nvtm;
        g = T0 + gmin;
        c = IVjmFwd - SatCurrent + T0 * (v - vjmFwd) + gmin * v;
    }
}

/* trap-assisted tunnelling factor of one junction component
 * (b4ld.c:911-980): T = exp(-v/Nvtmr * vts/(vts-v)) and dT/dv */
NGSF_HD inline void b4_tat(double vts, double Nvtmr, double v, double &T, double &dT)
{
    double T0, T9, T10;
    if ((vts - v) < (vts * 1e-3)) {
        T9 = 1.0e3;
        T0 = -v / Nvtmr * T9;
        b4_dexp(T0, T, T10);
        dT = T10 / Nvtmr * T9;
    } else {
        T9 = 1.0 / (vts - v);
        T0 = -v / Nvtmr * vts * T9;
        double dT0 = vts / Nvtmr * (T9 + v * T9 * T9);
        b4_dexp(T0, T, T10);
        dT = T10 * dT0;
    }
}

/* CONSTvt0: thermal voltage at the reference temperature 27 C
 * (const.h CONSTboltz * REFTEMP / CHARGE), the pnjlim scale of BSIM4. */
#define B4_CONSTVT0 (1.38064852e-23 * (27.0 + 273.15) / 1.6021766208e-19)

typedef DevCtx B4Ctx;

#include "bsim4_eval.cuh"

#endif
