/*
 * BSIM4 (level 54, 4.8.3) host setup: model defaults, temperature and
 * size-dependent parameters, junction and overlap constants, resolved per
 * instance into the B4P_* image the GPU load reads.
 *
 * Restates, for the selector subset the GPU load implements:
 *   BSIM4setup defaults           src/spicelib/devices/bsim4/b4set.c:60-2360
 *   BSIM4temp model/instance part src/spicelib/devices/bsim4/b4temp.c:79-2396
 *   BSIM4PAeffGeo                 src/spicelib/devices/bsim4/b4geo.c:25-150
 *   BSIM4checkModel value clamps  src/spicelib/devices/bsim4/b4check.c:290-600
 * Parameter names and defaults come from bsim4_params.def.
 */
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "bsim4.h"
#include "circuit.h"

namespace ngsf {

namespace {

enum B4Field {
#define B4F(f) MF_##f,
#define B4N(f, n)
#define B4D(f, v)
#define B4X(f, e)
#define B4BIN(f)
#include "bsim4_params.def"
#undef B4F
#undef B4N
#undef B4D
#undef B4X
#undef B4BIN
    MF_COUNT
};

struct NameEntry { const char *name; int field; };
const NameEntry kNames[] = {
#define B4F(f)
#define B4N(f, n) {n, MF_##f},
#define B4D(f, v)
#define B4X(f, e)
#define B4BIN(f)
#include "bsim4_params.def"
#undef B4F
#undef B4N
#undef B4D
#undef B4X
#undef B4BIN
};

/* constants of b4temp.c / b4ld.c */
const double kKb = 1.3806226e-23;
const double kKboQ = 8.617087e-5;
const double kEPS0 = 8.85418e-12;
const double kEPSSI = 1.03594e-10;
const double kPI = 3.141592654;
const double kMAX_EXP = 5.834617425e14;
const double kMIN_EXP = 1.713908431e-15;
const double kEXP_THRESHOLD = 34.0;
const double kCharge_q = 1.60219e-19;
const double kDELTA = 1.0e-9;
const double kCtoK = 273.15;
/* const.h: CONSTvt0 = CONSTboltz * REFTEMP / CHARGE, CONSTroot2 = sqrt 2 */
const double kCONSTvt0 = 1.38064852e-23 * (27.0 + kCtoK) / 1.6021766208e-19;
const double kCONSTroot2 = 1.4142135623730950488016887242097;

void dexp(double A, double &B)
{
    if (A > kEXP_THRESHOLD)
        B = kMAX_EXP * (1.0 + A - kEXP_THRESHOLD);
    else if (A < -kEXP_THRESHOLD)
        B = kMIN_EXP;
    else
        B = exp(A);
}

struct B4Model {
    double v[MF_COUNT];
    bool g[MF_COUNT];
    /* model-level temperature results (b4temp.c:79-418) */
    double epsrox, toxe, epssub, coxe, coxp, vcrit, factor1, vtm0, vtm, Eg0, ni;
    double SjctTempSatCurDensity, SjctSidewallTempSatCurDensity, SjctGateSidewallTempSatCurDensity;
    double DjctTempSatCurDensity, DjctSidewallTempSatCurDensity, DjctGateSidewallTempSatCurDensity;
    double SunitAreaTempJctCap, DunitAreaTempJctCap, SunitLengthSidewallTempJctCap;
    double DunitLengthSidewallTempJctCap, SunitLengthGateSidewallTempJctCap;
    double DunitLengthGateSidewallTempJctCap;
    double PhiBS, PhiBD, PhiBSWS, PhiBSWD, PhiBSWGS, PhiBSWGD;
    bool v47;   /* version 4.7.x: the reference's BSIM4v7 device */
};

#define M(f) (bm.v[MF_##f])
#define G(f) (bm.g[MF_##f])

void apply_defaults(B4Model &bm, double tnom_opt)
{
#define B4F(f)
#define B4N(f, n)
#define B4D(f, val) if (!G(f)) M(f) = (val);
#define B4X(f, e) if (!G(f)) M(f) = (e);
#define B4BIN(f)
#include "bsim4_params.def"
#undef B4F
#undef B4N
#undef B4D
#undef B4X
#undef B4BIN
    /* conditional defaults outside the plain pattern (b4set.c:2215-2290) */
    if (!G(njtsd)) M(njtsd) = G(njts) ? M(njts) : 20.0;
    if (!G(njtsswd)) M(njtsswd) = G(njtssw) ? M(njtssw) : 20.0;
    if (!G(njtsswgd)) M(njtsswgd) = G(njtsswg) ? M(njtsswg) : 20.0;
    if (!G(tnjtsd)) M(tnjtsd) = G(tnjts) ? M(tnjts) : 0.0;
    if (!G(tnjtsswd)) M(tnjtsswd) = G(tnjtssw) ? M(tnjtssw) : 0.0;
    if (!G(tnjtsswgd)) M(tnjtsswgd) = G(tnjtsswg) ? M(tnjtsswg) : 0.0;
}

void check_selectors(const B4Model &bm, const std::string &mname)
{
    auto need = [&](const char *what, double v, double want) {
        if (v != want)
            throw NetlistError("BSIM4 model " + mname + ": " + what + "=" +
                               std::to_string((int)v) + " is not supported by the GPU load (" +
                               what + "=" + std::to_string((int)want) + " only)");
    };
    need("mobmod", M(mobMod), 0);
    need("capmod", M(capMod), 2);
    need("rdsmod", M(rdsMod), 0);
    need("rbodymod", M(rbodyMod), 0);
    need("rgatemod", M(rgateMod), 0);
    need("trnqsmod", M(trnqsMod), 0);
    need("acnqsmod", M(acnqsMod), 0);
    need("igcmod", M(igcMod), 0);
    need("igbmod", M(igbMod), 0);
    need("diomod", M(dioMod), 1);
    need("tempmod", M(tempMod), 0);
    need("mtrlmod", M(mtrlMod), 0);
    need("gidlmod", M(gidlMod), 0);
    need("cvchargemod", M(cvchargeMod), 0);
    if (G(vtl) && M(vtl) > 0.0)
        throw NetlistError("BSIM4 model " + mname + ": vtl (source-end velocity limit) is not supported");
    if (G(lambda) && M(lambda) > 0.0)
        throw NetlistError("BSIM4 model " + mname + ": lambda (velocity overshoot) is not supported");
    if (M(wpemod) != 0)
        throw NetlistError("BSIM4 model " + mname + ": wpemod is not supported");
}

/* model part of BSIM4temp (b4temp.c:79-418) */
void model_temp(B4Model &bm, double Temp)
{
    if (M(SbulkJctPotential) < 0.1) M(SbulkJctPotential) = 0.1;
    if (M(SsidewallJctPotential) < 0.1) M(SsidewallJctPotential) = 0.1;
    if (M(SGatesidewallJctPotential) < 0.1) M(SGatesidewallJctPotential) = 0.1;
    if (M(DbulkJctPotential) < 0.1) M(DbulkJctPotential) = 0.1;
    if (M(DsidewallJctPotential) < 0.1) M(DsidewallJctPotential) = 0.1;
    if (M(DGatesidewallJctPotential) < 0.1) M(DGatesidewallJctPotential) = 0.1;

    /* BSIM4v7 defaults cf in setup, before the thickness consistency below
     * can change toxe (b4v7set.c:1908-1910); 4.8 defaults it after
     * (b4temp.c:173-175) */
    const double toxe_setup = M(toxe);
    /* mtrlMod 0 oxide thickness consistency */
    {
        double chktol = fabs(M(toxe));
        if (fabs(M(toxp)) > chktol) chktol = fabs(M(toxp));
        if (fabs(M(dtox)) > chktol) chktol = fabs(M(dtox));
        chktol = chktol * 1e-14;
        if (G(toxe) && G(toxp) && G(dtox) && (fabs(M(toxe) - (M(toxp) + M(dtox))) > chktol)) {
            /* dtox ignored */
        } else if (G(toxe) && !G(toxp)) {
            M(toxp) = M(toxe) - M(dtox);
        } else if (!G(toxe) && G(toxp)) {
            M(toxe) = M(toxp) + M(dtox);
            if (!G(toxm))
                M(toxm) = M(toxe);
        }
    }
    bm.epsrox = M(epsrox);
    bm.toxe = M(toxe);
    bm.epssub = kEPSSI;
    const double epsrox = bm.epsrox, toxe = bm.toxe, epssub = bm.epssub;
    if (!G(cf))
        M(cf) = 2.0 * epsrox * kEPS0 / kPI * log(1.0 + 0.4e-6 / (bm.v47 ? toxe_setup : toxe));
    bm.coxe = epsrox * kEPS0 / toxe;

    bm.coxp = M(epsrox) * kEPS0 / M(toxp);

    if (!G(cgdo)) {
        if (G(dlc) && (M(dlc) > 0.0))
            M(cgdo) = M(dlc) * bm.coxe - M(cgdl);
        else
            M(cgdo) = 0.6 * M(xj) * bm.coxe;
    }
    if (!G(cgso)) {
        if (G(dlc) && (M(dlc) > 0.0))
            M(cgso) = M(dlc) * bm.coxe - M(cgsl);
        else
            M(cgso) = 0.6 * M(xj) * bm.coxe;
    }
    if (!G(cgbo))
        M(cgbo) = 2.0 * M(dwc) * bm.coxe;

    const double Tnom = M(tnom);
    bm.vcrit = kCONSTvt0 * log(kCONSTvt0 / (kCONSTroot2 * 1.0e-14));
    bm.factor1 = sqrt(epssub / (epsrox * kEPS0) * toxe);
    const double Vtm0 = bm.vtm0 = kKboQ * Tnom;
    const double Eg0 = 1.16 - 7.02e-4 * Tnom * Tnom / (Tnom + 1108.0);
    bm.ni = 1.45e10 * (Tnom / 300.15) * sqrt(Tnom / 300.15) * exp(21.5565981 - Eg0 / (2.0 * Vtm0));
    bm.Eg0 = Eg0;
    bm.vtm = kKboQ * Temp;
    const double Eg = 1.16 - 7.02e-4 * Temp * Temp / (Temp + 1108.0);
    if (Temp != Tnom) {
        double T0 = Eg0 / Vtm0 - Eg / bm.vtm;
        double T1 = log(Temp / Tnom);
        double T2 = T0 + M(SjctTempExponent) * T1;
        double T3 = exp(T2 / M(SjctEmissionCoeff));
        bm.SjctTempSatCurDensity = M(SjctSatCurDensity) * T3;
        bm.SjctSidewallTempSatCurDensity = M(SjctSidewallSatCurDensity) * T3;
        bm.SjctGateSidewallTempSatCurDensity = M(SjctGateSidewallSatCurDensity) * T3;
        T2 = T0 + M(DjctTempExponent) * T1;
        T3 = exp(T2 / M(DjctEmissionCoeff));
        bm.DjctTempSatCurDensity = M(DjctSatCurDensity) * T3;
        bm.DjctSidewallTempSatCurDensity = M(DjctSidewallSatCurDensity) * T3;
        bm.DjctGateSidewallTempSatCurDensity = M(DjctGateSidewallSatCurDensity) * T3;
    } else {
        bm.SjctTempSatCurDensity = M(SjctSatCurDensity);
        bm.SjctSidewallTempSatCurDensity = M(SjctSidewallSatCurDensity);
        bm.SjctGateSidewallTempSatCurDensity = M(SjctGateSidewallSatCurDensity);
        bm.DjctTempSatCurDensity = M(DjctSatCurDensity);
        bm.DjctSidewallTempSatCurDensity = M(DjctSidewallSatCurDensity);
        bm.DjctGateSidewallTempSatCurDensity = M(DjctGateSidewallSatCurDensity);
    }
    if (bm.SjctTempSatCurDensity < 0.0) bm.SjctTempSatCurDensity = 0.0;
    if (bm.SjctSidewallTempSatCurDensity < 0.0) bm.SjctSidewallTempSatCurDensity = 0.0;
    if (bm.SjctGateSidewallTempSatCurDensity < 0.0) bm.SjctGateSidewallTempSatCurDensity = 0.0;
    if (bm.DjctTempSatCurDensity < 0.0) bm.DjctTempSatCurDensity = 0.0;
    if (bm.DjctSidewallTempSatCurDensity < 0.0) bm.DjctSidewallTempSatCurDensity = 0.0;
    if (bm.DjctGateSidewallTempSatCurDensity < 0.0) bm.DjctGateSidewallTempSatCurDensity = 0.0;

    const double delTemp = Temp - M(tnom);
    double T0 = M(tcj) * delTemp;
    if (T0 >= -1.0) {
        bm.SunitAreaTempJctCap = M(SunitAreaJctCap) * (1.0 + T0);
        bm.DunitAreaTempJctCap = M(DunitAreaJctCap) * (1.0 + T0);
    } else {
        bm.SunitAreaTempJctCap = M(SunitAreaJctCap) > 0.0 ? 0.0 : 0.0;
        bm.DunitAreaTempJctCap = M(DunitAreaJctCap) > 0.0 ? 0.0 : 0.0;
    }
    T0 = M(tcjsw) * delTemp;
    if (M(SunitLengthSidewallJctCap) < 0.0) M(SunitLengthSidewallJctCap) = 0.0;
    if (M(DunitLengthSidewallJctCap) < 0.0) M(DunitLengthSidewallJctCap) = 0.0;
    if (T0 >= -1.0) {
        bm.SunitLengthSidewallTempJctCap = M(SunitLengthSidewallJctCap) * (1.0 + T0);
        bm.DunitLengthSidewallTempJctCap = M(DunitLengthSidewallJctCap) * (1.0 + T0);
    } else {
        bm.SunitLengthSidewallTempJctCap = 0.0;
        bm.DunitLengthSidewallTempJctCap = 0.0;
    }
    T0 = M(tcjswg) * delTemp;
    if (T0 >= -1.0) {
        bm.SunitLengthGateSidewallTempJctCap = M(SunitLengthGateSidewallJctCap) * (1.0 + T0);
        bm.DunitLengthGateSidewallTempJctCap = M(DunitLengthGateSidewallJctCap) * (1.0 + T0);
    } else {
        bm.SunitLengthGateSidewallTempJctCap = 0.0;
        bm.DunitLengthGateSidewallTempJctCap = 0.0;
    }
    bm.PhiBS = M(SbulkJctPotential) - M(tpb) * delTemp;
    if (bm.PhiBS < 0.01) bm.PhiBS = 0.01;
    bm.PhiBD = M(DbulkJctPotential) - M(tpb) * delTemp;
    if (bm.PhiBD < 0.01) bm.PhiBD = 0.01;
    bm.PhiBSWS = M(SsidewallJctPotential) - M(tpbsw) * delTemp;
    if (bm.PhiBSWS < 0.01) bm.PhiBSWS = 0.01;
    bm.PhiBSWD = M(DsidewallJctPotential) - M(tpbsw) * delTemp;
    if (bm.PhiBSWD < 0.01) bm.PhiBSWD = 0.01;
    bm.PhiBSWGS = M(SGatesidewallJctPotential) - M(tpbswg) * delTemp;
    if (bm.PhiBSWGS < 0.01) bm.PhiBSWGS = 0.01;
    bm.PhiBSWGD = M(DGatesidewallJctPotential) - M(tpbswg) * delTemp;
    if (bm.PhiBSWGD < 0.01) bm.PhiBSWGD = 0.01;
    if (M(ijthdfwd) <= 0.0) M(ijthdfwd) = 0.0;
    if (M(ijthsfwd) <= 0.0) M(ijthsfwd) = 0.0;
    if (M(ijthdrev) <= 0.0) M(ijthdrev) = 0.0;
    if (M(ijthsrev) <= 0.0) M(ijthsrev) = 0.0;
    if (M(bvd) <= 0.0) M(bvd) = 0.0;
    if (M(bvs) <= 0.0) M(bvs) = 0.0;
}

/* BSIM4NumFingerDiff + BSIM4PAeffGeo (b4geo.c) */
void pa_eff_geo(double nf, int geo, int minSD, double Weffcj, double DMCG, double DMCI,
                double DMDG, double &Ps, double &Pd, double &As, double &Ad)
{
    double nuIntD = 0.0, nuEndD = 0.0, nuIntS = 0.0, nuEndS = 0.0;
    if (geo < 9) {
        int NF = (int)nf;
        if ((NF % 2) != 0) {
            nuEndD = nuEndS = 1.0;
            nuIntD = nuIntS = 2.0 * std::fmax((nf - 1.0) / 2.0, 0.0);
        } else if (minSD == 1) {
            nuEndD = 2.0;
            nuIntD = 2.0 * std::fmax((nf / 2.0 - 1.0), 0.0);
            nuEndS = 0.0;
            nuIntS = nf;
        } else {
            nuEndD = 0.0;
            nuIntD = nf;
            nuEndS = 2.0;
            nuIntS = 2.0 * std::fmax((nf / 2.0 - 1.0), 0.0);
        }
    }
    double T0 = DMCG + DMCI, T1 = DMCG + DMCG, T2 = DMDG + DMDG;
    double Piso = T0 + T0 + Weffcj, Psha = T1, Pmer = T2;
    double Aiso = T0 * Weffcj, Asha = DMCG * Weffcj, Amer = DMDG * Weffcj;
    switch (geo) {
    case 0: Ps = nuEndS * Piso + nuIntS * Psha; Pd = nuEndD * Piso + nuIntD * Psha;
            As = nuEndS * Aiso + nuIntS * Asha; Ad = nuEndD * Aiso + nuIntD * Asha; break;
    case 1: Ps = nuEndS * Piso + nuIntS * Psha; Pd = (nuEndD + nuIntD) * Psha;
            As = nuEndS * Aiso + nuIntS * Asha; Ad = (nuEndD + nuIntD) * Asha; break;
    case 2: Ps = (nuEndS + nuIntS) * Psha; Pd = nuEndD * Piso + nuIntD * Psha;
            As = (nuEndS + nuIntS) * Asha; Ad = nuEndD * Aiso + nuIntD * Asha; break;
    case 3: Ps = (nuEndS + nuIntS) * Psha; Pd = (nuEndD + nuIntD) * Psha;
            As = (nuEndS + nuIntS) * Asha; Ad = (nuEndD + nuIntD) * Asha; break;
    case 4: Ps = nuEndS * Piso + nuIntS * Psha; Pd = nuEndD * Pmer + nuIntD * Psha;
            As = nuEndS * Aiso + nuIntS * Asha; Ad = nuEndD * Amer + nuIntD * Asha; break;
    case 5: Ps = (nuEndS + nuIntS) * Psha; Pd = nuEndD * Pmer + nuIntD * Psha;
            As = (nuEndS + nuIntS) * Asha; Ad = nuEndD * Amer + nuIntD * Asha; break;
    case 6: Ps = nuEndS * Pmer + nuIntS * Psha; Pd = nuEndD * Piso + nuIntD * Psha;
            As = nuEndS * Amer + nuIntS * Asha; Ad = nuEndD * Aiso + nuIntD * Asha; break;
    case 7: Ps = nuEndS * Pmer + nuIntS * Psha; Pd = (nuEndD + nuIntD) * Psha;
            As = nuEndS * Amer + nuIntS * Asha; Ad = (nuEndD + nuIntD) * Asha; break;
    case 8: Ps = nuEndS * Pmer + nuIntS * Psha; Pd = nuEndD * Pmer + nuIntD * Psha;
            As = nuEndS * Amer + nuIntS * Asha; Ad = nuEndD * Amer + nuIntD * Asha; break;
    case 9: Ps = Piso + (nf - 1.0) * Psha; Pd = nf * Psha;
            As = Aiso + (nf - 1.0) * Asha; Ad = nf * Asha; break;
    case 10: Ps = nf * Psha; Pd = Piso + (nf - 1.0) * Psha;
             As = nf * Asha; Ad = Aiso + (nf - 1.0) * Asha; break;
    default:
        throw NetlistError("BSIM4: geomod " + std::to_string(geo) + " out of range");
    }
}

double ijth_vjm(double Nvtm, double Ijth, double Isb, double XExpBV)
{
    double Tc = XExpBV;
    double Tb = 1.0 + Ijth / Isb - Tc;
    double EVjmovNv = 0.5 * (Tb + sqrt(Tb * Tb + 4.0 * Tc));
    return Nvtm * log(EVjmovNv);
}

/* the last model resolved, so that consecutive instances of one model (and
 * per-device model cards of Monte Carlo decks) cost one model evaluation
 * without keeping every model's table alive; keyed by content */
struct ModelCache {
    bool valid = false;
    std::string name;
    int polarity = 0;
    std::map<std::string, double> params;
    double temp = 0, tnom = 0;
    B4Model bm;
};
thread_local ModelCache gCache;

const B4Model &resolve_model(const Model &m, double temp, double tnom_opt)
{
    ModelCache &mc = gCache;
    if (mc.valid && mc.name == m.name && mc.polarity == m.polarity && mc.temp == temp &&
        mc.tnom == tnom_opt && mc.params == m.p.v)
        return mc.bm;
    mc.valid = false;
    B4Model &bm = mc.bm;
    std::memset(&bm, 0, sizeof bm);
    M(type) = m.polarity;
    G(type) = true;
    bm.v47 = m.bsim4_v47();
    /* model parameters the BSIM4v7 device does not have (bsim4v7/b4v7.c):
     * its parser ignores them (parser/inpgmod.c:189) */
    static const char *kNotIn47[] = {"gidlclamp", "idovvdsc", "ketac", "lketac", "wketac",
                                     "pketac"};
    for (const auto &kv : m.p.v) {
        const std::string &k = kv.first;
        if (k == "level")
            continue;
        if (k == "version") {
            if (!bm.v47 && (kv.second < 4.8 - 1e-9 || kv.second >= 4.9))
                throw NetlistError("BSIM4 model " + m.name +
                                   ": only versions 4.7.x and 4.8.x are implemented (other "
                                   "versions select another device in the reference)");
            continue;
        }
        if (bm.v47) {
            bool skip = false;
            for (const char *x : kNotIn47)
                if (k == x)
                    skip = true;
            if (skip)
                continue;
            /* BSIM4v7 also has a model-level rgeomod (b4v7.c:137) */
            if (k == "rgeomod") {
                if (kv.second != 0.0)
                    throw NetlistError("BSIM4 model " + m.name +
                                       ": rgeomod=" + std::to_string((int)kv.second) +
                                       " is not supported by the GPU load (rgeomod=0 only)");
                continue;
            }
        }
        int field = -1;
        {
            /* name -> field, first table entry winning (a Monte Carlo deck
             * resolves one card per transistor) */
            static const std::unordered_map<std::string, int> index = [] {
                std::unordered_map<std::string, int> ix;
                for (const auto &ne : kNames)
                    ix.emplace(ne.name, ne.field);
                return ix;
            }();
            auto it = index.find(k);
            if (it != index.end())
                field = it->second;
        }
        if (field < 0)
            throw NetlistError("BSIM4 model " + m.name + ": unknown parameter '" + k + "'");
        double v = kv.second;
        /* unit conventions of b4mpar.c */
        if (field == MF_tnom)
            v = v + kCtoK;
        if ((field == MF_ndep || field == MF_lndep || field == MF_wndep || field == MF_pndep) && v > 1.0e20)
            v *= 1.0e-6;
        if ((field == MF_nsd || field == MF_lnsd || field == MF_wnsd || field == MF_pnsd ||
             field == MF_ngate || field == MF_lngate || field == MF_wngate || field == MF_pngate) &&
            v > 1.0e23)
            v *= 1.0e-6;
        bm.v[field] = v;
        bm.g[field] = true;
    }
    apply_defaults(bm, tnom_opt);
    check_selectors(bm, m.name);
    model_temp(bm, temp);
    mc.valid = true;
    mc.name = m.name;
    mc.polarity = m.polarity;
    mc.params = m.p.v;
    mc.temp = temp;
    mc.tnom = tnom_opt;
    return bm;
}

}  // namespace

/* Resolve one BSIM4 instance.  p receives B4P_COUNT values; needDp/needSp
 * report whether series resistance needs internal drain/source nodes
 * (b4set.c:2437-2530). */
void bsim4_params(const Circuit &c, const Model &m, const Instance &in, double *p,
                  bool &needDp, bool &needSp)
{
    const B4Model &bmc = resolve_model(m, c.opt.temp, c.opt.tnom);
    B4Model bm = bmc;   /* pParam and checkModel work on a private copy */
    const Params &ip = in.p;
    for (const auto &kv : ip.v) {
        static const char *known[] = {"l", "w", "m", "nf", "ad", "as", "pd", "ps", "nrd", "nrs",
                                      "off", "delvto", "mulu0", "min", "geomod", "sa", "sb", "sd",
                                      "mult_i", "mult_q"};
        bool ok = false;
        for (const char *k : known)
            if (kv.first == k)
                ok = true;
        if (!ok)
            throw NetlistError("BSIM4 instance " + in.name + ": parameter '" + kv.first +
                               "' is not supported");
        /* the BSIM4v7 instance table has no current/charge multipliers
         * (bsim4v7/b4v7.c): its parser rejects them (parser/inpdpar.c:130) */
        if (bm.v47 && (kv.first == "mult_i" || kv.first == "mult_q"))
            throw NetlistError("BSIM4 instance " + in.name + ": unknown parameter (" +
                               kv.first + ") for a version 4.7 model");
    }
    const double scale = 1.0;
    const double L = ip.has("l") ? ip.get("l", 0) * scale : 5.0e-6;
    const double W = ip.has("w") ? ip.get("w", 0) * scale : 5.0e-6;
    const double mm = ip.get("m", 1.0);
    const double mult_i = ip.get("mult_i", 1.0);
    const double mult_q = ip.get("mult_q", 1.0);
    const double nf = ip.get("nf", 1.0);
    const int minSD = (int)ip.get("min", 0.0);
    const int geoMod = ip.has("geomod") ? (int)ip.get("geomod", 0) : (int)M(geoMod);
    const double delvto = ip.get("delvto", 0.0);
    const double mulu0 = ip.get("mulu0", 1.0);
    const double sa = ip.get("sa", 0.0), sb = ip.get("sb", 0.0);
    if (sa > 0.0 && sb > 0.0)
        throw NetlistError("BSIM4 instance " + in.name + ": layout stress (sa/sb) is not supported");
    const bool off = ip.has("off");

    /* series resistance nodes: rdsMod 0, rgeoMod 0 (b4set.c:2437-2530) */
    needDp = (M(sheetResistance) > 0) && ip.has("nrd") && ip.get("nrd", 1.0) > 0;
    needSp = (M(sheetResistance) > 0) && ip.has("nrs") && ip.get("nrs", 1.0) > 0;

    const double Temp = c.opt.temp;
    const double Tnom = M(tnom);
    const double TRatio = Temp / Tnom;
    const double delTemp = Temp - M(tnom);
    const double epsrox = bm.epsrox, toxe = bm.toxe, epssub = bm.epssub;
    const double Vtm0 = bm.vtm0;
    const double Eg0 = bm.Eg0;
    const double ni = bm.ni;

    /* ---- size-dependent parameters (b4temp.c:421-1655) ---- */
    double pp[MF_COUNT];   /* pParam values, indexed like the model fields */
    std::memcpy(pp, bm.v, sizeof pp);
#define PP(f) (pp[MF_##f])
    const double Ldrn = L;
    const double Lnew = L + M(xl);
    const double Wnew = W / nf + M(xw);
    double T0 = pow(Lnew, M(Lln));
    double T1 = pow(Wnew, M(Lwn));
    double tmp1 = M(Ll) / T0 + M(Lw) / T1 + M(Lwl) / (T0 * T1);
    const double dl = M(Lint) + tmp1;
    double tmp2 = M(Llc) / T0 + M(Lwc) / T1 + M(Lwlc) / (T0 * T1);
    const double dlc = M(dlc) + tmp2;
    double T2 = pow(Lnew, M(Wln));
    double T3 = pow(Wnew, M(Wwn));
    tmp1 = M(Wl) / T2 + M(Ww) / T3 + M(Wwl) / (T2 * T3);
    const double dw = M(Wint) + tmp1;
    tmp2 = M(Wlc) / T2 + M(Wwc) / T3 + M(Wwlc) / (T2 * T3);
    const double dwc = M(dwc) + tmp2;
    const double dwj = M(dwj) + tmp2;
    const double leff = Lnew - 2.0 * dl;
    if (leff <= 0.0)
        throw NetlistError("BSIM4 " + in.name + ": effective channel length <= 0");
    const double weff = Wnew - 2.0 * dw;
    if (weff <= 0.0)
        throw NetlistError("BSIM4 " + in.name + ": effective channel width <= 0");
    const double leffCV = Lnew - 2.0 * dlc;
    if (leffCV <= 0.0)
        throw NetlistError("BSIM4 " + in.name + ": effective channel length for C-V <= 0");
    const double weffCV = Wnew - 2.0 * dwc;
    if (weffCV <= 0.0)
        throw NetlistError("BSIM4 " + in.name + ": effective channel width for C-V <= 0");
    const double weffCJ = Wnew - 2.0 * dwj;
    if (weffCJ <= 0.0)
        throw NetlistError("BSIM4 " + in.name + ": effective channel width for S/D junctions <= 0");
    double Inv_L, Inv_W, Inv_LW;
    if (M(binUnit) == 1) {
        Inv_L = 1.0e-6 / leff;
        Inv_W = 1.0e-6 / weff;
        Inv_LW = 1.0e-12 / (leff * weff);
    } else {
        Inv_L = 1.0 / leff;
        Inv_W = 1.0 / weff;
        Inv_LW = 1.0 / (leff * weff);
    }
#define B4F(f)
#define B4N(f, n)
#define B4D(f, v)
#define B4X(f, e)
#define B4BIN(f) PP(f) = M(f) + M(l##f) * Inv_L + M(w##f) * Inv_W + M(p##f) * Inv_LW;
#include "bsim4_params.def"
#undef B4F
#undef B4N
#undef B4D
#undef B4X
#undef B4BIN

    const double abulkCVfactor = 1.0 + pow((PP(clc) / leffCV), PP(cle));
    T0 = (TRatio - 1.0);
    const double PowWeffWr = pow(weffCJ * 1.0e6, PP(wr)) * nf;
    PP(ucs) = PP(ucs) * pow(TRatio, PP(ucste));
    /* tempMod 0 */
    PP(ua) = PP(ua) + PP(ua1) * T0;
    PP(ub) = PP(ub) + PP(ub1) * T0;
    PP(uc) = PP(uc) + PP(uc1) * T0;
    PP(ud) = PP(ud) + PP(ud1) * T0;
    double vsattemp = PP(vsat) - PP(at) * T0;
    double T10 = PP(prt) * T0;
    double rds0 = (PP(rdsw) + T10) * nf / PowWeffWr;
    double rdswmin = (M(rdswmin) + T10) * nf / PowWeffWr;
    if (PP(u0) > 1.0)
        PP(u0) = PP(u0) / 1.0e4;
    double T5 = 1.0 - PP(up) * exp(-leff / PP(lp));
    double u0temp = PP(u0) * T5 * pow(TRatio, PP(ute));
    if (PP(eu) < 0.0) PP(eu) = 0.0;
    if (PP(ucs) < 0.0) PP(ucs) = 0.0;
    PP(vfbsdoff) = PP(vfbsdoff) * (1.0 + PP(tvfbsdoff) * delTemp);
    PP(voff) = PP(voff) * (1.0 + PP(tvoff) * delTemp);
    PP(nfactor) = PP(nfactor) + PP(tnfactor) * delTemp / Tnom;
    /* BSIM4v7 never bins tvoffcv, so its size-dependent copy stays 0
     * (b4v7temp.c:1267; 4.8 bins it at b4temp.c:868-871) */
    if (bm.v47)
        PP(tvoffcv) = 0.0;
    PP(voffcv) = PP(voffcv) * (1.0 + PP(tvoffcv) * delTemp);
    PP(eta0) = PP(eta0) + PP(teta0) * delTemp / Tnom;

    const double cgdo_p = (M(cgdo) + PP(cf)) * weffCV;
    const double cgso_p = (M(cgso) + PP(cf)) * weffCV;
    const double cgbo_p = M(cgbo) * leffCV * nf;

    if (!G(ndep) && G(gamma1)) {
        T0 = PP(gamma1) * bm.coxe;
        PP(ndep) = 3.01248e22 * T0 * T0;
    }
    const double phi = Vtm0 * log(PP(ndep) / ni) + PP(phin) + 0.4;
    if (phi <= 0.0)
        throw NetlistError("BSIM4 " + in.name + ": phi <= 0 (check phin and ndep)");
    const double sqrtPhi = sqrt(phi);
    const double Xdep0 = sqrt(2.0 * epssub / (kCharge_q * PP(ndep) * 1.0e6)) * sqrtPhi;
    const double litl = sqrt(3.0 * 3.9 / epsrox * PP(xj) * toxe);
    const double vbi = Vtm0 * log(PP(nsd) * PP(ndep) / (ni * ni));
    const double cdep0 = sqrt(kCharge_q * epssub * PP(ndep) * 1.0e6 / 2.0 / phi);
    const double mstar = 0.5 + atan(PP(minv)) / kPI;
    const double voffcbn = PP(voff) + M(voffl) / leff;
    const double ldeb = sqrt(epssub * Vtm0 / (kCharge_q * PP(ndep) * 1.0e6)) / 3.0;
    const double acde = PP(acde) * pow((PP(ndep) / 2.0e16), -0.25);

    double k1 = PP(k1), k2 = PP(k2), vbx = PP(vbx), vbm = PP(vbm);
    if (G(k1) || G(k2)) {
        if (!G(k1)) k1 = 0.53;
        if (!G(k2)) k2 = -0.0186;
    } else {
        if (!G(vbx))
            vbx = phi - 7.7348e-4 * PP(ndep) * PP(xt) * PP(xt);
        if (vbx > 0.0) vbx = -vbx;
        if (vbm > 0.0) vbm = -vbm;
        double gamma1 = PP(gamma1), gamma2 = PP(gamma2);
        if (!G(gamma1)) gamma1 = 5.753e-12 * sqrt(PP(ndep)) / bm.coxe;
        if (!G(gamma2)) gamma2 = 5.753e-12 * sqrt(PP(nsub)) / bm.coxe;
        T0 = gamma1 - gamma2;
        T1 = sqrt(phi - vbx) - sqrtPhi;
        T2 = sqrt(phi * (phi - vbm)) - phi;
        k2 = T0 * T1 / (2.0 * T2 + vbm);
        k1 = gamma2 - 2.0 * k2 * sqrt(phi - vbm);
    }
    double vfb = PP(vfb), vth0 = PP(vth0);
    if (!G(vfb)) {
        if (G(vth0))
            vfb = M(type) * vth0 - phi - k1 * sqrtPhi;
        else
            vfb = -1.0;
    }
    if (!G(vth0))
        vth0 = M(type) * (vfb + phi + k1 * sqrtPhi);
    const double k1ox = k1 * toxe / M(toxm);

    double tmp = sqrt(epssub / (epsrox * kEPS0) * toxe * Xdep0);
    T0 = PP(dsub) * leff / tmp;
    double theta0vb0;
    if (T0 < kEXP_THRESHOLD) {
        T1 = exp(T0);
        T2 = T1 - 1.0;
        T3 = T2 * T2;
        double T4 = T3 + 2.0 * T1 * kMIN_EXP;
        theta0vb0 = T1 / T4;
    } else {
        theta0vb0 = 1.0 / (kMAX_EXP - 2.0);
    }
    T0 = PP(drout) * leff / tmp;
    if (T0 < kEXP_THRESHOLD) {
        T1 = exp(T0);
        T2 = T1 - 1.0;
        T3 = T2 * T2;
        double T4 = T3 + 2.0 * T1 * kMIN_EXP;
        T5 = T1 / T4;
    } else {
        T5 = 1.0 / (kMAX_EXP - 2.0);
    }
    const double thetaRout = PP(pdibl1) * T5 + PP(pdibl2);

    tmp = sqrt(Xdep0);
    tmp1 = vbi - phi;
    tmp2 = bm.factor1 * tmp;
    T0 = PP(dvt1w) * weff * leff / tmp2;
    double T8;
    if (T0 < kEXP_THRESHOLD) {
        T1 = exp(T0);
        T2 = T1 - 1.0;
        T3 = T2 * T2;
        double T4 = T3 + 2.0 * T1 * kMIN_EXP;
        T8 = T1 / T4;
    } else {
        T8 = 1.0 / (kMAX_EXP - 2.0);
    }
    T0 = PP(dvt0w) * T8;
    T8 = T0 * tmp1;
    T0 = PP(dvt1) * leff / tmp2;
    double T9;
    if (T0 < kEXP_THRESHOLD) {
        T1 = exp(T0);
        T2 = T1 - 1.0;
        T3 = T2 * T2;
        double T4 = T3 + 2.0 * T1 * kMIN_EXP;
        T9 = T1 / T4;
    } else {
        T9 = 1.0 / (kMAX_EXP - 2.0);
    }
    T9 = PP(dvt0) * T9 * tmp1;
    double T4 = toxe * phi / (weff + PP(w0));
    T0 = sqrt(1.0 + PP(lpe0) / leff);
    T3 = (PP(kt1) + PP(kt1l) / leff) * (TRatio - 1.0);
    T5 = k1ox * (T0 - 1.0) * sqrtPhi + T3;
    const double vfbzbfactor = -T8 - T9 + PP(k3) * T4 + T5 - phi - k1 * sqrtPhi;

    /* stress effect: only the reference values (sa = sb = 0) */
    {
        double wlod = M(wlod);
        if (M(wlod) < 0.0) wlod = 0.0;
        (void)wlod;
    }
    /* DITS_Sft2 factor (b4temp.c:1650-1652) */
    T0 = -PP(dvtp3) * log(leff);
    dexp(T0, T1);
    const double dvtp2factor = PP(dvtp5) + PP(dvtp2) * T1;

    /* BSIM4checkModel clamps that change values the load reads */
    if (PP(ckappas) < 0.02) PP(ckappas) = 0.02;
    if (PP(ckappad) < 0.02) PP(ckappad) = 0.02;
    if (PP(a2) < 0.01) {
        PP(a2) = 0.01;
    } else if (PP(a2) > 1.0) {
        PP(a2) = 1.0;
        PP(a1) = 0.0;
    }
    if (PP(prwg) < 0.0) PP(prwg) = 0.0;
    if (PP(rdsw) < 0.0) {
        PP(rdsw) = 0.0;
        rds0 = 0.0;
    }
    if (rds0 < 0.0) rds0 = 0.0;
    if (rdswmin < 0.0) rdswmin = 0.0;

    /* ---- instance part (b4temp.c:1656-2260) ---- */
    double inst_vth0 = vth0;
    double inst_k2 = k2;
    double inst_eta0 = PP(eta0);
    inst_vth0 += delvto;
    const double inst_vfb = vfb + M(type) * delvto;
    u0temp = u0temp * mulu0;
    T3 = M(type) * inst_vth0 - inst_vfb - phi;
    const double vtfbphi2 = (4.0 * T3 < 0.0) ? 0.0 : 4.0 * T3;
    double vbsc;
    if (inst_k2 < 0.0) {
        T0 = 0.5 * k1 / inst_k2;
        vbsc = 0.9 * (phi - T0 * T0);
        if (vbsc > -3.0)
            vbsc = -3.0;
        else if (vbsc < -30.0)
            vbsc = -30.0;
    } else {
        vbsc = -30.0;
    }
    if (vbsc > vbm)
        vbsc = vbm;
    const double k2ox = inst_k2 * toxe / M(toxm);
    const double vfbzb = vfbzbfactor + M(type) * inst_vth0;

    const double DMCGeff = M(dmcg) - M(dmcgt);
    const double DMCIeff = M(dmci);
    const double DMDGeff = M(dmdg) - M(dmcgt);
    double Pseff, Pdeff, Aseff, Adeff, dumPs, dumPd, dumAs, dumAd;
    if (ip.has("ps")) {
        double v = ip.get("ps", 0) * scale;
        if (v == 0.0) Pseff = 0.0;
        else if (v < 0.0) Pseff = 0.0;
        else Pseff = M(perMod) == 0 ? v : v - weffCJ * nf;
    } else {
        pa_eff_geo(nf, geoMod, minSD, weffCJ, DMCGeff, DMCIeff, DMDGeff, Pseff, dumPd, dumAs, dumAd);
    }
    if (Pseff < 0.0) Pseff = 0.0;
    if (ip.has("pd")) {
        double v = ip.get("pd", 0) * scale;
        if (v == 0.0) Pdeff = 0.0;
        else if (v < 0.0) Pdeff = 0.0;
        else Pdeff = M(perMod) == 0 ? v : v - weffCJ * nf;
    } else {
        pa_eff_geo(nf, geoMod, minSD, weffCJ, DMCGeff, DMCIeff, DMDGeff, dumPs, Pdeff, dumAs, dumAd);
    }
    if (Pdeff < 0.0) Pdeff = 0.0;
    if (ip.has("as"))
        Aseff = ip.get("as", 0) * scale * scale;
    else
        pa_eff_geo(nf, geoMod, minSD, weffCJ, DMCGeff, DMCIeff, DMDGeff, dumPs, dumPd, Aseff, dumAd);
    if (Aseff < 0.0) Aseff = 0.0;
    if (ip.has("ad"))
        Adeff = ip.get("ad", 0) * scale * scale;
    else
        pa_eff_geo(nf, geoMod, minSD, weffCJ, DMCGeff, DMCIeff, DMDGeff, dumPs, dumPd, dumAs, Adeff);
    if (Adeff < 0.0) Adeff = 0.0;

    double sourceConductance = 0.0, drainConductance = 0.0;
    if (needSp) {
        sourceConductance = M(sheetResistance) * ip.get("nrs", 1.0);
        sourceConductance = sourceConductance > 0.0 ? 1.0 / sourceConductance : 1.0e3;
    }
    if (needDp) {
        drainConductance = M(sheetResistance) * ip.get("nrd", 1.0);
        drainConductance = drainConductance > 0.0 ? 1.0 / drainConductance : 1.0e3;
    }

    /* junction saturation currents, dioMod 1 (b4temp.c:2107-2225) */
    const double Nvtms = bm.vtm * M(SjctEmissionCoeff);
    double SourceSatCurrent;
    if ((Aseff <= 0.0) && (Pseff <= 0.0))
        SourceSatCurrent = 0.0;
    else
        SourceSatCurrent = Aseff * bm.SjctTempSatCurDensity + Pseff * bm.SjctSidewallTempSatCurDensity +
                           weffCJ * nf * bm.SjctGateSidewallTempSatCurDensity;
    double vjsmFwd = 0.0, IVjsmFwd = 0.0;
    if (SourceSatCurrent > 0.0) {
        vjsmFwd = ijth_vjm(Nvtms, M(ijthsfwd), SourceSatCurrent, 0.0);
        IVjsmFwd = SourceSatCurrent * exp(vjsmFwd / Nvtms);
    }
    const double Nvtmd = bm.vtm * M(DjctEmissionCoeff);
    double DrainSatCurrent;
    if ((Adeff <= 0.0) && (Pdeff <= 0.0))
        DrainSatCurrent = 0.0;
    else
        DrainSatCurrent = Adeff * bm.DjctTempSatCurDensity + Pdeff * bm.DjctSidewallTempSatCurDensity +
                          weffCJ * nf * bm.DjctGateSidewallTempSatCurDensity;
    double vjdmFwd = 0.0, IVjdmFwd = 0.0;
    if (DrainSatCurrent > 0.0) {
        vjdmFwd = ijth_vjm(Nvtmd, M(ijthdfwd), DrainSatCurrent, 0.0);
        IVjdmFwd = DrainSatCurrent * exp(vjdmFwd / Nvtmd);
    }

    /* trap-assisted tunnelling constants (b4temp.c:2228-2261) */
    T0 = (TRatio - 1.0);
    const double njtsstemp = M(njts) * (1.0 + M(tnjts) * T0);
    const double njtsswstemp = M(njtssw) * (1.0 + M(tnjtssw) * T0);
    const double njtsswgstemp = M(njtsswg) * (1.0 + M(tnjtsswg) * T0);
    const double njtsdtemp = M(njtsd) * (1.0 + M(tnjtsd) * T0);
    const double njtsswdtemp = M(njtsswd) * (1.0 + M(tnjtsswd) * T0);
    const double njtsswgdtemp = M(njtsswgd) * (1.0 + M(tnjtsswgd) * T0);
    const double T7 = Eg0 / bm.vtm * T0;
    double E1, E2, E3, E4, E5, E6;
    dexp(M(xtss) * T7, E1);
    dexp(M(xtsd) * T7, E2);
    dexp(M(xtssws) * T7, E3);
    dexp(M(xtsswd) * T7, E4);
    dexp(M(xtsswgs) * T7, E5);
    dexp(M(xtsswgd) * T7, E6);
    double jtweff = M(jtweff) < 0.0 ? 0.0 : M(jtweff);
    const double T11 = sqrt(jtweff / weffCJ) + 1.0;
    T10 = weffCJ * nf;

    /* junction capacitance constants (b4ld.c:3947-3962) */
    const double czbd = bm.DunitAreaTempJctCap * Adeff;
    const double czbs = bm.SunitAreaTempJctCap * Aseff;
    const double czbdsw = bm.DunitLengthSidewallTempJctCap * Pdeff;
    const double czbdswg = bm.DunitLengthGateSidewallTempJctCap * weffCJ * nf;
    const double czbssw = bm.SunitLengthSidewallTempJctCap * Pseff;
    const double czbsswg = bm.SunitLengthGateSidewallTempJctCap * weffCJ * nf;

    double *o = p;
#define SET(f, val) o[B4P_##f] = (val)
    SET(type, M(type));
    SET(off, off ? 1.0 : 0.0);
    SET(icVDS, 0.0);
    SET(icVGS, 0.0);
    SET(icVBS, 0.0);
    SET(vth0, inst_vth0);
    SET(vcrit, bm.vcrit);
    SET(vtm, bm.vtm);
    SET(vtm0, bm.vtm0);
    SET(SourceSatCurrent, SourceSatCurrent);
    SET(DrainSatCurrent, DrainSatCurrent);
    SET(Nvtms, Nvtms);
    SET(Nvtmd, Nvtmd);
    SET(vjsmFwd, vjsmFwd);
    SET(IVjsmFwd, IVjsmFwd);
    SET(vjdmFwd, vjdmFwd);
    SET(IVjdmFwd, IVjdmFwd);
    SET(Nvtmrss, bm.vtm0 * njtsstemp);
    SET(Nvtmrssws, bm.vtm0 * njtsswstemp);
    SET(Nvtmrsswgs, bm.vtm0 * njtsswgstemp);
    SET(Nvtmrsd, bm.vtm0 * njtsdtemp);
    SET(Nvtmrsswd, bm.vtm0 * njtsswdtemp);
    SET(Nvtmrsswgd, bm.vtm0 * njtsswgdtemp);
    SET(vtss, M(vtss));
    SET(vtssws, M(vtssws));
    SET(vtsswgs, M(vtsswgs));
    SET(vtsd, M(vtsd));
    SET(vtsswd, M(vtsswd));
    SET(vtsswgd, M(vtsswgd));
    SET(SjctTempRevSatCur, E1 * Aseff * M(jtss));
    SET(DjctTempRevSatCur, E2 * Adeff * M(jtsd));
    SET(SswTempRevSatCur, E3 * Pseff * M(jtssws));
    SET(DswTempRevSatCur, E4 * Pdeff * M(jtsswd));
    SET(SswgTempRevSatCur, E5 * T10 * T11 * M(jtsswgs));
    SET(DswgTempRevSatCur, E6 * T10 * T11 * M(jtsswgd));
    SET(vbsc, vbsc);
    SET(phi, phi);
    SET(Xdep0, Xdep0);
    SET(sqrtPhi, sqrtPhi);
    SET(factor1, bm.factor1);
    SET(vbi, vbi);
    SET(dvt2, PP(dvt2));
    SET(dvt2w, PP(dvt2w));
    SET(dvt1, PP(dvt1));
    SET(leff, leff);
    SET(dvt0, PP(dvt0));
    SET(dvt1w, PP(dvt1w));
    SET(weff, weff);
    SET(dvt0w, PP(dvt0w));
    SET(tempRatio, Temp / M(tnom) - 1.0);
    SET(lpe0, PP(lpe0));
    SET(k1ox, k1ox);
    SET(kt1, PP(kt1));
    SET(kt1l, PP(kt1l));
    SET(kt2, PP(kt2));
    SET(toxe, toxe);
    SET(w0, PP(w0));
    SET(eta0, inst_eta0);
    SET(etab, PP(etab));
    SET(theta0vb0, theta0vb0);
    SET(lpeb, PP(lpeb));
    SET(k1, k1);
    SET(k2ox, k2ox);
    SET(k3, PP(k3));
    SET(k3b, PP(k3b));
    SET(coxe, bm.coxe);
    SET(cit, PP(cit));
    SET(nfactor, PP(nfactor));
    SET(cdsc, PP(cdsc));
    SET(cdscb, PP(cdscb));
    SET(cdscd, PP(cdscd));
    SET(dvtp0, PP(dvtp0));
    SET(dvtp1, PP(dvtp1));
    SET(dvtp4, PP(dvtp4));
    SET(dvtp2factor, dvtp2factor);
    SET(vfb, inst_vfb);
    SET(ngate, PP(ngate));
    SET(mstar, mstar);
    SET(voffcbn, voffcbn);
    SET(cdep0, cdep0);
    SET(dwg, PP(dwg));
    SET(dwb, PP(dwb));
    SET(prwg, PP(prwg));
    SET(prwb, PP(prwb));
    SET(rds0, rds0);
    SET(rdswmin, rdswmin);
    SET(nf, nf);
    SET(xj, PP(xj));
    SET(a0, PP(a0));
    SET(b0, PP(b0));
    SET(b1, PP(b1));
    SET(ags, PP(ags));
    SET(keta, PP(keta));
    SET(ketac, PP(ketac));
    SET(ua, PP(ua));
    SET(uc, PP(uc));
    SET(ub, PP(ub));
    SET(ud, PP(ud));
    SET(u0temp, u0temp);
    SET(vsattemp, vsattemp);
    SET(a1, PP(a1));
    SET(a2, PP(a2));
    SET(delta, PP(delta));
    SET(vtfbphi2, vtfbphi2);
    SET(toxp, M(toxp));
    SET(coxp, bm.coxp);
    SET(bdos, M(bdos));
    SET(ados, M(ados));
    SET(fprout, PP(fprout));
    SET(pvag, PP(pvag));
    SET(pclm, PP(pclm));
    SET(litl, litl);
    SET(thetaRout, thetaRout);
    SET(pdiblb, PP(pdiblb));
    SET(pditsd, PP(pditsd));
    SET(pdits, PP(pdits));
    SET(pditsl, M(pditsl));
    SET(pscbe1, PP(pscbe1));
    SET(pscbe2, PP(pscbe2));
    SET(alpha0, PP(alpha0));
    SET(alpha1, PP(alpha1));
    SET(beta0, PP(beta0));
    SET(egidl, PP(egidl));
    SET(agidl, PP(agidl));
    SET(bgidl, PP(bgidl));
    SET(cgidl, PP(cgidl));
    SET(weffCJ, weffCJ);
    SET(egisl, PP(egisl));
    SET(agisl, PP(agisl));
    SET(bgisl, PP(bgisl));
    SET(cgisl, PP(cgisl));
    SET(abulkCVfactor, abulkCVfactor);
    SET(weffCV, weffCV);
    SET(leffCV, leffCV);
    SET(noff, PP(noff));
    SET(voffcv, PP(voffcv));
    SET(vfbzb, vfbzb);
    SET(acde, acde);
    SET(ldeb, ldeb);
    SET(moin, PP(moin));
    SET(xpart, M(xpart));
    SET(cgdo, cgdo_p);
    SET(cgso, cgso_p);
    SET(cgbo, cgbo_p);
    SET(cgdl, PP(cgdl));
    SET(cgsl, PP(cgsl));
    SET(ckappad, PP(ckappad));
    SET(ckappas, PP(ckappas));
    SET(czbd, czbd);
    SET(czbs, czbs);
    SET(czbdsw, czbdsw);
    SET(czbdswg, czbdswg);
    SET(czbssw, czbssw);
    SET(czbsswg, czbsswg);
    SET(MJS, M(SbulkJctBotGradingCoeff));
    SET(MJSWS, M(SbulkJctSideGradingCoeff));
    SET(MJSWGS, M(SbulkJctGateSideGradingCoeff));
    SET(MJD, M(DbulkJctBotGradingCoeff));
    SET(MJSWD, M(DbulkJctSideGradingCoeff));
    SET(MJSWGD, M(DbulkJctGateSideGradingCoeff));
    SET(PhiBS, bm.PhiBS);
    SET(PhiBSWS, bm.PhiBSWS);
    SET(PhiBSWGS, bm.PhiBSWGS);
    SET(PhiBD, bm.PhiBD);
    SET(PhiBSWD, bm.PhiBSWD);
    SET(PhiBSWGD, bm.PhiBSWGD);
    SET(drainConductance, drainConductance);
    SET(sourceConductance, sourceConductance);
    SET(m, mm);
    SET(mult_i, mult_i * mm);
    SET(mult_q, mult_q * mm);
    SET(version47, bm.v47 ? 1.0 : 0.0);
#undef SET
#undef PP
    (void)kKb;
    (void)kDELTA;
    (void)Ldrn;
    (void)vbx;
}

#undef M
#undef G

}  // namespace ngsf
