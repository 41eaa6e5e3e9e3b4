/*
 * Junction diode (DIO, level 1) image shared by the host compiler
 * (dio_setup.cpp) and the load (dio_eval.cuh): per-instance values in
 * structure-of-arrays layout, field f of instance i at p[f * n + i].
 */
#ifndef NGSF_DIO_H
#define NGSF_DIO_H

/* terminals: anode, cathode, and the anode side of the series resistance
 * (equal to the anode when rs = 0; src/spicelib/devices/dio/diosetup.c) */
enum { DIN_POS, DIN_NEG, DIN_POSP, DIN_COUNT };

#define DIP_LIST(X)                                                           \
    X(vte) X(vtebrk) X(tSatCur) X(tVcrit) X(tBrkdwnV) X(bvGiven) X(gspr)      \
    X(tJctCap) X(tJctPot) X(tDepCap) X(tGradingCoeff) X(tF1) X(tF2) X(tF3)     \
    X(tJctSWCap) X(tJctSWPot) X(tDepSWCap) X(gradingSWCoeff) X(tF2SW)          \
    X(tF3SW) X(tTransitTime) X(ikf) X(ikfGiven) X(ikr) X(ikrGiven) X(off)      \
    X(capMP)

#define DIP_ENUM(f) DIP_##f,
enum { DIP_LIST(DIP_ENUM) DIP_COUNT };
#undef DIP_ENUM

/* state vector layout (diodefs.h DIOvoltage .. DIOgqcsr, 22 doubles) */
enum {
    DIS_VOLTAGE = 0, DIS_CURRENT = 1, DIS_CONDUCT = 2, DIS_CAPCHARGE = 6,
    DIS_CAPCURRENT = 7, DIS_QTH = 10, DIS_DELTEMP = 12, DIS_DIDIO_DT = 13,
    DIS_SRCAPCHARGE = 15, DIS_QP = 17, DIS_RESCURRENT = 18, DIS_RESCONDUCT = 19,
    DIS_CQCSR = 20, DIS_GQCSR = 21, DIS_COUNT = 22
};

/* stamps in DIOload order (dioload.c:785-815): rhs neg, rhs pos', then
 * pos-pos, neg-neg, pos'-pos', pos-pos', neg-pos', pos'-pos, pos'-neg */
#define DIO_NSTAMP 9

#endif
