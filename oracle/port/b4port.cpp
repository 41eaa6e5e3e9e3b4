/*
 * Test infrastructure: BSIM4 for the CPU oracle port.
 *
 * The port restates the reference's transient control flow, matrix
 * assembly and solver independently; the BSIM4 model arithmetic itself
 * (BSIM4setup/BSIM4temp, src/spicelib/devices/bsim4/b4set.c, b4temp.c, and
 * BSIM4load, b4ld.c) is the product's own host-callable evaluation,
 * compiled here for the CPU.  Its correctness is pinned separately by the
 * golden fixtures generated with the reference build (tests/golden).
 * Nothing in the product links this file.
 */
#include <cstring>
#include <string>

#include "../../ngspice-sf-mirror_gb300/csrc/bsim4_load.cuh"
#include "../../ngspice-sf-mirror_gb300/csrc/dio_eval.cuh"
#include "../../ngspice-sf-mirror_gb300/csrc/circuit.h"

extern "C" int port_b4_nparam(void) { return B4P_COUNT; }
extern "C" int port_b4_nstate(void) { return B4S_COUNT; }
extern "C" int port_b4_nstamp(void) { return B4_NSTAMP; }

/* Resolve one instance: model card (name, polarity, key/value pairs) and
 * instance parameters -> B4P_COUNT values.  Returns 0, or -1 with err. */
extern "C" int port_b4_params(const char *mname, int polarity, int nm, const char **mkeys,
                              const double *mvals, const char *iname, int ni,
                              const char **ikeys, const double *ivals, double temp,
                              double tnom, double *out, int *needDp, int *needSp, char *err,
                              int errlen)
{
    try {
        ngsf::Circuit c;
        c.opt.temp = temp;
        c.opt.tnom = tnom;
        ngsf::Model m;
        m.name = mname;
        m.kind = ngsf::K_BSIM4;
        m.polarity = polarity;
        for (int k = 0; k < nm; k++)
            m.p.v[mkeys[k]] = mvals[k];
        ngsf::Instance in;
        in.name = iname;
        in.kind = ngsf::K_BSIM4;
        for (int k = 0; k < ni; k++)
            in.p.v[ikeys[k]] = ivals[k];
        bool dp = false, sp = false;
        ngsf::bsim4_params(c, m, in, out, dp, sp);
        *needDp = dp;
        *needSp = sp;
        return 0;
    } catch (const std::exception &e) {
        if (err && errlen > 0) {
            std::strncpy(err, e.what(), (size_t)errlen - 1);
            err[errlen - 1] = 0;
        }
        return -1;
    }
}

/* One instance load; sv receives B4_NSTAMP stamp values. */
extern "C" int port_b4_load_one(int mode, int order, int gear, double gmin, double delta,
                                double deltaOld1, double ag0, double ag1, double ag2,
                                const double *rhsOld, double *st0, double *st1,
                                const double *st2, const double *p, double *h, const int *node,
                                int st, double *sv)
{
    B4Ctx x;
    x.mode = mode;
    x.order = order;
    x.gear = gear;
    x.gmin = gmin;
    x.delta = delta;
    x.deltaOld1 = deltaOld1;
    x.ag0 = ag0;
    x.ag1 = ag1;
    x.ag2 = ag2;
    x.rhsOld = rhsOld;
    x.st0 = st0;
    x.st1 = st1;
    x.st2 = st2;
    return bsim4_eval(x, p, 1, h, 1, node, st, sv, 1);
}

/* stamp pattern: (row, col) as B4N_* terminal indices, row -1 = rhs */
extern "C" void port_b4_pattern(int *rows, int *cols)
{
    enum { D = B4N_D, G = B4N_G, S = B4N_S, B = B4N_B, DP = B4N_DP, SP = B4N_SP };
    static const int pat[B4_NSTAMP][2] = {
        {-1, DP}, {-1, G}, {-1, B}, {-1, SP},
        {G, G}, {G, DP}, {G, SP}, {G, B},
        {DP, DP}, {DP, D}, {DP, G}, {DP, SP}, {DP, B}, {D, DP}, {D, D},
        {SP, DP}, {SP, G}, {SP, SP}, {SP, S}, {SP, B}, {S, SP}, {S, S},
        {B, DP}, {B, G}, {B, SP}, {B, B},
        {DP, DP}, {DP, G}, {DP, SP}, {DP, B}, {B, DP}, {B, G}, {B, SP}, {B, B},
        {SP, DP}, {SP, G}, {SP, SP}, {SP, B}, {B, DP}, {B, G}, {B, SP}, {B, B}};
    for (int k = 0; k < B4_NSTAMP; k++) {
        rows[k] = pat[k][0];
        cols[k] = pat[k][1];
    }
}

/* ---------------- junction diode (shared evaluation, as above) -------- */
extern "C" int port_dio_nparam(void) { return DIP_COUNT; }
extern "C" int port_dio_nstate(void) { return DIS_COUNT; }

extern "C" int port_dio_params(const char *mname, int nm, const char **mkeys, const double *mvals,
                               const char *iname, int ni, const char **ikeys, const double *ivals,
                               double temp, double tnom, double reltol, double *out,
                               int *needPosPrime, char *err, int errlen)
{
    try {
        ngsf::Circuit c;
        c.opt.temp = temp;
        c.opt.tnom = tnom;
        c.opt.reltol = reltol;
        ngsf::Model m;
        m.name = mname;
        m.kind = ngsf::K_DIO;
        for (int k = 0; k < nm; k++)
            m.p.v[mkeys[k]] = mvals[k];
        ngsf::Instance in;
        in.name = iname;
        in.kind = ngsf::K_DIO;
        for (int k = 0; k < ni; k++)
            in.p.v[ikeys[k]] = ivals[k];
        bool pp = false;
        ngsf::dio_params(c, m, in, out, pp);
        *needPosPrime = pp;
        return 0;
    } catch (const std::exception &e) {
        if (err && errlen > 0) {
            std::strncpy(err, e.what(), (size_t)errlen - 1);
            err[errlen - 1] = 0;
        }
        return -1;
    }
}

extern "C" int port_dio_load_one(int mode, int order, int gear, double gmin, double delta,
                                 double deltaOld1, double ag0, double ag1, double ag2,
                                 const double *rhsOld, double *st0, double *st1,
                                 const double *st2, const double *p, const int *node, int st,
                                 double *sv)
{
    DevCtx x;
    x.mode = mode;
    x.order = order;
    x.gear = gear;
    x.gmin = gmin;
    x.delta = delta;
    x.deltaOld1 = deltaOld1;
    x.ag0 = ag0;
    x.ag1 = ag1;
    x.ag2 = ag2;
    x.rhsOld = rhsOld;
    x.st0 = st0;
    x.st1 = st1;
    x.st2 = st2;
    return dio_eval(x, p, 1, node, st, sv, 1);
}
