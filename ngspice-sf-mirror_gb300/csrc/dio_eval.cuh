/*
 * Junction diode load (DIOload, src/spicelib/devices/dio/dioload.c:17-865)
 * for level 1 without sidewall diode, self-heating, soft reverse recovery,
 * tunnelling or recombination currents (rejected at compile time), bypass
 * off, PREDICTOR undefined.  Host- and device-callable; one instance per
 * call, stamps written to sv[k * svs] in the order of DIO_NSTAMP.
 */
#ifndef NGSF_DIO_EVAL_CUH
#define NGSF_DIO_EVAL_CUH

#include <math.h>
#include <stddef.h>

#include "devsup.cuh"
#include "dio.h"
#include "ngsf_types.h"

/* CONSTe (const.h CONSTnap) */
#define DIO_CONSTE 2.7182818284590452353602874713527

NGSF_HD inline int dio_eval(const DevCtx &x, const double *P, size_t ps, const int *node, int st,
                            double *sv, size_t svs)
{
#define DQ(f) P[(size_t)DIP_##f * ps]
    const int mode = x.mode;
    double *st0 = x.st0 + st;
    double *st1 = x.st1 + st;
    const double *st2 = x.st2 + st;
    const bool off = DQ(off) != 0.0;
    const double vte = DQ(vte), vtebrk = DQ(vtebrk);
    const double gspr = DQ(gspr);
    const double tVcrit = DQ(tVcrit), tBrkdwnV = DQ(tBrkdwnV);
    const bool bvGiven = DQ(bvGiven) != 0.0;
    int Check_dio = 1;
    double vd;

    /* initialisation, prediction and limiting (dioload.c:100-335) */
    if (mode & NGSF_MODEINITTRAN) {
        vd = st1[DIS_VOLTAGE];
    } else if ((mode & NGSF_MODEINITJCT) && off) {
        vd = 0;
    } else if (mode & NGSF_MODEINITJCT) {
        vd = tVcrit;
    } else if ((mode & NGSF_MODEINITFIX) && off) {
        vd = 0;
    } else {
        if (mode & NGSF_MODEINITPRED) {
            st0[DIS_VOLTAGE] = st1[DIS_VOLTAGE];
            vd = dev_pred(x, st1, st2, DIS_VOLTAGE);
            st0[DIS_CURRENT] = st1[DIS_CURRENT];
            st0[DIS_CONDUCT] = st1[DIS_CONDUCT];
            st0[DIS_DELTEMP] = st1[DIS_DELTEMP];
            st0[DIS_DIDIO_DT] = st1[DIS_DIDIO_DT];
            st0[DIS_QTH] = st1[DIS_QTH];
            st0[DIS_RESCURRENT] = st1[DIS_RESCURRENT];
            st0[DIS_RESCONDUCT] = st1[DIS_RESCONDUCT];
            st0[DIS_CQCSR] = st1[DIS_CQCSR];
            st0[DIS_GQCSR] = st1[DIS_GQCSR];
            if (mode & NGSF_MODEGUESS)   /* predictor guess in rhsOld */
                vd = x.rhsOld[node[DIN_POSP]] - x.rhsOld[node[DIN_NEG]];
        } else {
            vd = x.rhsOld[node[DIN_POSP]] - x.rhsOld[node[DIN_NEG]];
            st0[DIS_QTH] = 0.0;   /* cth0 * delTemp, no self-heating */
        }
        if (bvGiven && (vd < NG_MIN(0, -tBrkdwnV + 10 * vtebrk))) {
            double vdtemp = -(vd + tBrkdwnV);
            vdtemp = dev_pnjlim(vdtemp, -(st0[DIS_VOLTAGE] + tBrkdwnV), vtebrk, tVcrit, &Check_dio);
            vd = -(vdtemp + tBrkdwnV);
        } else {
            vd = dev_pnjlim(vd, st0[DIS_VOLTAGE], vte, tVcrit, &Check_dio);
        }
    }

    /* dc current and conductance (dioload.c:345-500) */
    const double csat = DQ(tSatCur);
    double cdb, gdb;
    if (vd >= -3 * vte) {
        double evd = exp(vd / vte);
        cdb = csat * (evd - 1);
        gdb = csat * evd / vte;
    } else if ((!bvGiven) || vd >= -tBrkdwnV) {
        double arg = 3 * vte / (vd * DIO_CONSTE);
        arg = arg * arg * arg;
        cdb = -csat * (1 + arg);
        gdb = csat * 3 * arg / vd;
    } else {
        double evrev = exp(-(tBrkdwnV + vd) / vtebrk);
        cdb = -csat * evrev;
        gdb = csat * evrev / vtebrk;
    }
    if (vd >= -3 * vte) {
        if ((DQ(ikfGiven) != 0.0) && (cdb > 1.0e-18)) {
            const double ikf = DQ(ikf);
            double sq = sqrt(cdb / ikf);
            gdb = ((1 + sq) * gdb - cdb * gdb / (2 * sq * ikf)) / (1 + 2 * sq + cdb / ikf);
            cdb = cdb / (1 + sq);
        }
    } else {
        if ((DQ(ikrGiven) != 0.0) && (cdb < -1.0e-18)) {
            const double ikr = DQ(ikr);
            double sq = sqrt(cdb / (-ikr));
            gdb = ((1 + sq) * gdb + cdb * gdb / (2 * sq * ikr)) / (1 + 2 * sq - cdb / ikr);
            cdb = cdb / (1 + sq);
        }
    }
    double cd = cdb + x.gmin * vd;
    double gd = gdb + x.gmin;
    const double cdres = cd, gdres = gd;

    /* charge storage (dioload.c:520-690) */
    if (mode & (NGSF_MODEDCTRANCURVE | NGSF_MODETRAN)) {
        const double czero = DQ(tJctCap), tJctPot = DQ(tJctPot), tDepCap = DQ(tDepCap);
        const double tGrad = DQ(tGradingCoeff);
        double deplcharge, deplcap;
        if (vd < tDepCap) {
            double arg = 1 - vd / tJctPot;
            double sarg = exp(-tGrad * log(arg));
            deplcharge = tJctPot * czero * (1 - arg * sarg) / (1 - tGrad);
            deplcap = czero * sarg;
        } else {
            double czof2 = czero / DQ(tF2);
            deplcharge = czero * DQ(tF1) +
                         czof2 * (DQ(tF3) * (vd - tDepCap) +
                                  (tGrad / (tJctPot + tJctPot)) * (vd * vd - tDepCap * tDepCap));
            deplcap = czof2 * (DQ(tF3) + tGrad * vd / tJctPot);
        }
        const double czeroSW = DQ(tJctSWCap), tJctSWPot = DQ(tJctSWPot);
        const double gradSW = DQ(gradingSWCoeff), tDepSWCap = DQ(tDepSWCap);
        double deplchargeSW, deplcapSW;
        if (vd < tDepSWCap) {
            double argSW = 1 - vd / tJctSWPot;
            double sargSW = exp(-gradSW * log(argSW));
            deplchargeSW = tJctSWPot * czeroSW * (1 - argSW * sargSW) / (1 - gradSW);
            deplcapSW = czeroSW * sargSW;
        } else {
            double czof2SW = czeroSW / DQ(tF2SW);
            deplchargeSW = czeroSW * DQ(tF1) +
                           czof2SW * (DQ(tF3SW) * (vd - tDepSWCap) +
                                      (gradSW / (tJctSWPot + tJctSWPot)) *
                                          (vd * vd - tDepSWCap * tDepSWCap));
            deplcapSW = czof2SW * (DQ(tF3SW) + gradSW * vd / tJctSWPot);
        }
        const double tt = DQ(tTransitTime), cmp = DQ(capMP);
        double diffcharge = tt * cd;
        double diffcap = tt * gd;
        st0[DIS_CAPCHARGE] = diffcharge + deplcharge + deplchargeSW + cmp * vd;
        double capd = diffcap + deplcap + deplcapSW + cmp;
        st0[DIS_SRCAPCHARGE] = 0;
        if (mode & NGSF_MODEINITTRAN)
            st1[DIS_CAPCHARGE] = st0[DIS_CAPCHARGE];
        dev_integrate(x, st0, st1, st2, DIS_CAPCHARGE);
        gd = gd + x.ag0 * capd;
        cd = cd + st0[DIS_CAPCURRENT];
        if (mode & NGSF_MODEINITTRAN)
            st1[DIS_CAPCURRENT] = st0[DIS_CAPCURRENT];
    }

    /* convergence flag and state (dioload.c:697-740) */
    int noncon = 0;
    if ((!(mode & NGSF_MODEINITFIX)) || (!off))
        if (Check_dio == 1)
            noncon = 1;
    st0[DIS_VOLTAGE] = vd;
    st0[DIS_CURRENT] = cd;
    st0[DIS_CONDUCT] = gd;
    st0[DIS_DELTEMP] = 0.0;
    st0[DIS_DIDIO_DT] = 0.0;
    st0[DIS_QP] = 0.0;
    st0[DIS_RESCURRENT] = cdres;
    st0[DIS_RESCONDUCT] = gdres;
    st0[DIS_CQCSR] = 0.0;
    st0[DIS_GQCSR] = 0.0;

    /* stamps (dioload.c:785-815) */
    const double cdeq = cd - gd * vd;
    sv[0 * svs] = cdeq;
    sv[1 * svs] = -cdeq;
    sv[2 * svs] = gspr;
    sv[3 * svs] = gd;
    sv[4 * svs] = gd + gspr;
    sv[5 * svs] = -gspr;
    sv[6 * svs] = -gd;
    sv[7 * svs] = -gspr;
    sv[8 * svs] = -gd;
#undef DQ
    return noncon;
}

#endif
