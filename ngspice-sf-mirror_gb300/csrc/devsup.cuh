/*
 * Newton voltage limiting shared by the device loads
 * (src/spicelib/devices/devsup.c: DEVlimvds :21, DEVpnjlim :50,
 * DEVfetlim :93).  Host- and device-callable so that the same model
 * arithmetic can be checked on the CPU.
 */
#ifndef NGSF_DEVSUP_CUH
#define NGSF_DEVSUP_CUH

#include <math.h>

#ifdef __CUDACC__
#define NGSF_HD __host__ __device__
#else
#define NGSF_HD
#endif

/* MIN / MAX exactly as the reference macros (src/include/ngspice/macros.h) */
#ifndef NG_MAX
#define NG_MAX(a, b) ((a) > (b) ? (a) : (b))
#define NG_MIN(a, b) ((a) < (b) ? (a) : (b))
#endif

NGSF_HD inline double dev_limvds(double vnew, double vold)
{
    if (vold >= 3.5) {
        if (vnew > vold)
            vnew = NG_MIN(vnew, (3 * vold) + 2);
        else if (vnew < 3.5)
            vnew = NG_MAX(vnew, 2);
    } else {
        if (vnew > vold)
            vnew = NG_MIN(vnew, 4);
        else
            vnew = NG_MAX(vnew, -.5);
    }
    return vnew;
}

NGSF_HD inline double dev_pnjlim(double vnew, double vold, double vt, double vcrit, int *icheck)
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

NGSF_HD inline double dev_fetlim(double vnew, double vold, double vto)
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
                    vnew = NG_MAX(vnew, vto + 2);
                }
            } else {
                if (delv >= vtsthi)
                    vnew = vold + vtsthi;
            }
        } else {
            if (delv <= 0)
                vnew = NG_MAX(vnew, vto - .5);
            else
                vnew = NG_MIN(vnew, vto + 4);
        }
    } else {
        if (delv <= 0) {
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
    }
    return vnew;
}

/* DEVqmeyer: Meyer gate capacitances (devsup.c:674-736) */

/* Iteration context a device load reads besides its own instance:
 * CKTmode, CKTorder, CKTintegrateMethod (gear), CKTgmin, CKTdelta,
 * CKTdeltaOld[1], CKTag[0..2], CKTrhsOld and the state vectors
 * CKTstate0..2. */
struct DevCtx {
    int mode;
    int order;
    int gear;
    double gmin, delta, deltaOld1, ag0, ag1, ag2;
    const double *rhsOld;
    double *st0;
    double *st1;
    const double *st2;
};

/* NIintegrate (src/maths/ni/niinteg.c:18-80) for a charge at state offset
 * q whose current lives at q+1 (st0..st2: this instance's CKTstate0..2).
 * Trapezoidal orders 1 and 2; Gear sums ag[order]*q_order down to
 * ag[0]*q_0 from zero, in that order. */
NGSF_HD inline double ni_integ_current(int gear, int order, double ag0, double ag1, double ag2,
                                       const double *st0, const double *st1,
                                       const double *st2, int q)
{
    if (gear) {
        double c = 0;
        if (order >= 2)
            c += ag2 * st2[q];
        c += ag1 * st1[q];
        c += ag0 * st0[q];
        return c;
    }
    if (order == 1)
        return ag0 * st0[q] + ag1 * st1[q];
    return -st1[q + 1] * ag1 + ag0 * (st0[q] - st1[q]);
}

NGSF_HD inline void dev_integrate(const DevCtx &x, double *st0, const double *st1,
                                  const double *st2, int q)
{
    st0[q + 1] = ni_integ_current(x.gear, x.order, x.ag0, x.ag1, x.ag2, st0, st1, st2, q);
}

/* DEVpred (src/spicelib/devices/devsup.c:815-827): linear extrapolation of
 * a state from the two previous time points */
NGSF_HD inline double dev_pred(const DevCtx &x, const double *st1, const double *st2, int q)
{
    double xfact = x.delta / x.deltaOld1;
    return ((1 + xfact) * st1[q]) - (xfact * st2[q]);
}

#endif
