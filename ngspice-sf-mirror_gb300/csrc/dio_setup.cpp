/*
 * Junction diode host setup: model defaults (DIOsetup,
 * src/spicelib/devices/dio/diosetup.c:30-330), temperature update
 * (DIOtempUpdate, diotemp.c:20-280) and the instance values the load reads.
 * Level 1 only; the parts of the model the GPU load does not implement
 * (sidewall diode with its own resistance or current, self-heating, soft
 * reverse recovery, tunnelling, recombination current, tlev/tlevc other
 * than 0) are refused with a message.
 */
#include <cmath>
#include <string>

#include "circuit.h"
#include "dio.h"

namespace ngsf {

namespace {
const double kBoltz = 1.38064852e-23;     /* const.h CONSTboltz */
const double kCharge = 1.6021766208e-19;  /* const.h CHARGE */
const double kCtoK = 273.15;
const double kRefTemp = 27.0 + kCtoK;     /* const.h REFTEMP */
const double kKoverQ = kBoltz / kCharge;  /* CONSTKoverQ */
const double kRoot2 = 1.4142135623730950488016887242097;

struct Alias { const char *name, *field; };
/* netlist names of the supported model parameters (dio.c DIOmPTable) */
const Alias kNames[] = {
    {"level", "level"}, {"is", "is"}, {"js", "is"}, {"tnom", "tnom"}, {"tref", "tnom"},
    {"rs", "rs"}, {"trs", "trs1"}, {"trs1", "trs1"}, {"trs2", "trs2"}, {"n", "n"},
    {"tt", "tt"}, {"ttt1", "ttt1"}, {"ttt2", "ttt2"}, {"cjo", "cjo"}, {"cj0", "cjo"},
    {"cj", "cjo"}, {"vj", "vj"}, {"pb", "vj"}, {"m", "mj"}, {"mj", "mj"}, {"tm1", "tm1"},
    {"tm2", "tm2"}, {"cjp", "cjsw"}, {"cjsw", "cjsw"}, {"php", "vjsw"}, {"vjsw", "vjsw"},
    {"mjsw", "mjsw"}, {"ikf", "ikf"}, {"ik", "ikf"}, {"ikr", "ikr"}, {"nbv", "nbv"},
    {"nz", "nbv"}, {"area", "area"}, {"pj", "pj"}, {"tlev", "tlev"}, {"tlevc", "tlevc"},
    {"eg", "eg"}, {"xti", "xti"}, {"kf", "kf"}, {"af", "af"}, {"fc", "fc"}, {"fcs", "fcs"},
    {"bv", "bv"}, {"vb", "bv"}, {"vrb", "bv"}, {"var", "bv"}, {"ibv", "ibv"}, {"ib", "ibv"},
    {"tcv", "tcv"}, {"tbv1", "tcv"}, {"gap1", "gap1"}, {"gap2", "gap2"}, {"cta", "cta"},
    {"ctc", "cta"}, {"ctp", "ctp"}, {"tpb", "tpb"}, {"tvj", "tpb"}, {"tphp", "tphp"},
    {"fv_max", "-"}, {"bv_max", "-"}, {"id_max", "-"},
    {"te_max", "-"}, {"pd_max", "-"},
};
}  // namespace

/* p receives DIP_COUNT values; needPosPrime reports the series-resistance
 * node (diosetup.c:375-392). */
void dio_params(const Circuit &c, const Model &m, const Instance &in, double *p,
                bool &needPosPrime)
{
    Params mp;
    for (const auto &kv : m.p.v) {
        const char *field = nullptr;
        for (const auto &a : kNames)
            if (kv.first == a.name)
                field = a.field;
        if (!field)
            throw NetlistError("diode model " + m.name + ": parameter '" + kv.first +
                               "' is not supported by the GPU load");
        if (std::string(field) != "-")
            mp.v[field] = kv.second;
    }
    auto G = [&](const char *k) { return mp.has(k); };
    auto V = [&](const char *k, double d) { return mp.get(k, d); };
    if (G("level") && V("level", 1) != 1)
        throw NetlistError("diode model " + m.name + ": only level 1 is supported");
    /* temperature equation selectors (diotemp.c:59-238): tlev 0, 1, 2 and
     * tlevc 0, 1 */
    const int tlev = (int)V("tlev", 0), tlevc = (int)V("tlevc", 0);
    if (tlev < 0 || tlev > 2 || tlevc < 0 || tlevc > 1)
        throw NetlistError("diode model " + m.name + ": tlev " + std::to_string(tlev) +
                           " / tlevc " + std::to_string(tlevc) +
                           " are not supported (tlev 0-2, tlevc 0-1)");

    /* DIOsetup defaults */
    const double N = V("n", 1);
    double satCur = V("is", 1e-14);
    const double bvCur = V("ibv", 1e-3);
    const double jctPot = V("vj", 1);
    const double grading = V("mj", .5);
    const double gradT1 = V("tm1", 0.0), gradT2 = V("tm2", 0.0);
    const double fc = V("fc", .5), fcs = V("fcs", .5);
    const double tt = V("tt", 0), ttt1 = V("ttt1", 0.0), ttt2 = V("ttt2", 0.0);
    const double cjo = V("cjo", 0.0);
    const double cjsw = V("cjsw", 0);
    const double jctSWPot = V("vjsw", 1);
    const double gradSW = V("mjsw", .33);
    const bool ikfGiven = G("ikf") && V("ikf", 0) >= 1e-28;   /* CKTepsmin */
    const bool ikrGiven = G("ikr") && V("ikr", 0) >= 1e-28;
    const double brkN = V("nbv", N);
    const double eg = V("eg", 1.11);
    const double xti = V("xti", 3);
    const double tcv = V("tcv", 0.0);
    /* DIOsetup defaults of the tlev 2 band-gap and tlevc 1 coefficients
     * (diosetup.c:147-166) */
    const double gap1 = V("gap1", 7.02e-4), gap2 = V("gap2", 1108.0);
    const double cta = V("cta", 0.0), ctp = V("ctp", 0.0);
    const double tpb = V("tpb", 0.0), tphp = V("tphp", 0.0);
    const double areaModel = V("area", 1.0), pjModel = V("pj", 0.0);
    if (satCur < 1e-28)
        satCur = 1e-28;
    const double tnom = G("tnom") ? V("tnom", 0) + kCtoK : c.opt.tnom;
    const double rs = V("rs", 0);
    const double conductance = (!G("rs") || rs == 0) ? 0.0 : 1 / rs;
    const double trs1 = V("trs1", 0.0), trs2 = V("trs2", 0.0);

    /* instance */
    const Params &ip = in.p;
    for (const auto &kv : ip.v)
        if (kv.first != "area" && kv.first != "pj" && kv.first != "m" && kv.first != "off")
            throw NetlistError("diode " + in.name + ": parameter '" + kv.first +
                               "' is not supported");
    const double area = ip.has("area") ? ip.get("area", 1) : areaModel;
    const double pj = ip.has("pj") ? ip.get("pj", 0) : pjModel;
    const double mm = ip.get("m", 1);
    const double junctionCap = cjo * area * mm;
    const double junctionSWCap = cjsw * pj * mm;

    /* DIOtempUpdate at the circuit temperature */
    const double Temp = c.opt.temp;
    const double vt = kKoverQ * Temp;
    const double vte = N * vt;
    const double vtnom = kKoverQ * tnom;
    const double dt = Temp - tnom;
    const double lnTRatio = log(Temp / tnom);
    double factor = 1.0 + (gradT1 * dt) + (gradT2 * dt * dt);
    const double tGrading = grading * factor;
    double egfet, egfet1;
    if (tlev < 2) {
        egfet = 1.16 - (7.02e-4 * Temp * Temp) / (Temp + 1108);
        egfet1 = 1.16 - (7.02e-4 * tnom * tnom) / (tnom + 1108);
    } else {
        egfet = eg - (gap1 * Temp * Temp) / (Temp + gap2);
        egfet1 = eg - (gap1 * tnom * tnom) / (tnom + gap2);
    }
    const double fact2 = Temp / kRefTemp;
    const double arg = -egfet / (2 * kBoltz * Temp) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
    const double pbfact = -2 * vt * (1.5 * log(fact2) + kCharge * arg);
    const double arg1 = -egfet1 / (kBoltz * 2 * tnom) + 1.1150877 / (2 * kBoltz * kRefTemp);
    const double fact1 = tnom / kRefTemp;
    const double pbfact1 = -2 * vtnom * (1.5 * log(fact1) + kCharge * arg1);
    double tJctCap, tJctPot, tJctSWCap, tJctSWPot;
    if (tlevc == 0) {
        const double pbo = (jctPot - pbfact1) / fact1;
        const double gmaold = (jctPot - pbo) / pbo;
        tJctCap = junctionCap / (1 + tGrading * (400e-6 * (tnom - kRefTemp) - gmaold));
        tJctPot = pbfact + fact2 * pbo;
        const double gmanew = (tJctPot - pbo) / pbo;
        tJctCap *= 1 + tGrading * (400e-6 * (Temp - kRefTemp) - gmanew);
        const double pboSW = (jctSWPot - pbfact1) / fact1;
        const double gmaSWold = (jctSWPot - pboSW) / pboSW;
        tJctSWCap = junctionSWCap / (1 + gradSW * (400e-6 * (tnom - kRefTemp) - gmaSWold));
        tJctSWPot = pbfact + fact2 * pboSW;
        const double gmaSWnew = (tJctSWPot - pboSW) / pboSW;
        tJctSWCap *= 1 + gradSW * (400e-6 * (Temp - kRefTemp) - gmaSWnew);
    } else {
        /* linear in the distance from the reference temperature */
        tJctPot = jctPot - tpb * (Temp - kRefTemp);
        tJctCap = junctionCap * (1 + cta * (Temp - kRefTemp));
        tJctSWPot = jctSWPot - tphp * (Temp - kRefTemp);
        tJctSWCap = junctionSWCap * (1 + ctp * (Temp - kRefTemp));
    }
    double tSatCur;
    if (tlev < 2) {
        const double a1 = ((Temp / tnom) - 1) * eg / vte;
        const double a2 = xti / N * lnTRatio;
        tSatCur = satCur * area * mm * exp(a1 + a2);
    } else {
        /* band-gap form: Eg(Tnom) / (N vt(Tnom)) - Eg(T) / (N vt(T)) */
        const double a0 = egfet1 / (N * vtnom);
        const double a1 = egfet / vte;
        const double a2 = xti / N * lnTRatio;
        tSatCur = satCur * area * mm * exp(a0 - a1 + a2);
    }
    const double xfc = log(1 - fc);
    const double xfcs = log(1 - fcs);
    const double tF1 = tJctPot * (1 - exp((1 - tGrading) * xfc)) / (1 - tGrading);
    const double tDepCap = fc * tJctPot;
    const double tDepSWCap = fcs * tJctSWPot;
    const double totalSatCur = tSatCur + 0.0;
    const double tVcrit = vte * log(vte / (kRoot2 * totalSatCur));
    double tBrkdwnV = 0.0;
    if (G("bv")) {
        double tBV = tlev == 0 ? V("bv", 0) - tcv * dt : V("bv", 0) * (1 - tcv * dt);
        double cbv = mm * bvCur;
        double xbv;
        if (cbv < totalSatCur * tBV / vt) {
            xbv = tBV;
        } else {
            double tol = c.opt.reltol * cbv;
            xbv = tBV - brkN * vt * log(1 + cbv / totalSatCur);
            for (int iter = 0; iter < 25; iter++) {
                xbv = tBV - brkN * vt * log(cbv / totalSatCur + 1 - xbv / vt);
                double xcbv = totalSatCur * (exp((tBV - xbv) / (brkN * vt)) - 1 + xbv / vt);
                if (fabs(xcbv - cbv) <= tol)
                    break;
            }
        }
        tBrkdwnV = xbv;
    }
    factor = 1.0 + (ttt1 * dt) + (ttt2 * dt * dt);
    const double tTransitTime = tt * factor;
    double tConductance = conductance * area * mm;
    if (G("rs") && rs != 0.0) {
        factor = 1.0 + trs1 * dt + (trs2 * dt * dt);
        tConductance = conductance * area * mm / factor;
    }
    const double tF2 = exp((1 + tGrading) * xfc);
    const double tF3 = 1 - fc * (1 + tGrading);
    const double tF2SW = exp((1 + gradSW) * xfcs);
    const double tF3SW = 1 - fcs * (1 + gradSW);

    needPosPrime = rs != 0;
    double *o = p;
#define SET(f, val) o[DIP_##f] = (val)
    SET(vte, vte);
    SET(vtebrk, brkN * vt);
    SET(tSatCur, tSatCur);
    SET(tVcrit, tVcrit);
    SET(tBrkdwnV, tBrkdwnV);
    SET(bvGiven, G("bv") ? 1.0 : 0.0);
    SET(gspr, tConductance);
    SET(tJctCap, tJctCap);
    SET(tJctPot, tJctPot);
    SET(tDepCap, tDepCap);
    SET(tGradingCoeff, tGrading);
    SET(tF1, tF1);
    SET(tF2, tF2);
    SET(tF3, tF3);
    SET(tJctSWCap, tJctSWCap);
    SET(tJctSWPot, tJctSWPot);
    SET(tDepSWCap, tDepSWCap);
    SET(gradingSWCoeff, gradSW);
    SET(tF2SW, tF2SW);
    SET(tF3SW, tF3SW);
    SET(tTransitTime, tTransitTime);
    SET(ikf, V("ikf", 0) * area * mm);
    SET(ikfGiven, ikfGiven ? 1.0 : 0.0);
    SET(ikr, V("ikr", 0) * area * mm);
    SET(ikrGiven, ikrGiven ? 1.0 : 0.0);
    SET(off, ip.has("off") ? 1.0 : 0.0);
    SET(capMP, 0.0);
#undef SET
}

}  // namespace ngsf
