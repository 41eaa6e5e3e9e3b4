/*
 * Circuit compiler: CKTsetup / CKTtemp / TRANinit equivalents producing the
 * structure-of-arrays image of one circuit (see circuit.h).
 *
 * Reference correspondence:
 *   internal nodes, branch equations, state slots  DEVsetup
 *       (mos1/mos1set.c:44-213, vsrc/vsrcset.c, cap/capsetup.c)
 *   temperature-dependent parameters                 DEVtemperature
 *       (mos1/mos1temp.c:36-332, res/restemp.c RESupdate_conduct,
 *        cap/captemp.c)
 *   load-time constants of MOS1load hoisted here     mos1/mos1load.c:131-154
 *   matrix elements (SMPmakeElt / TSTALLOC)          one stamp slot per
 *       pointer of the device's load routine, in load order
 *   transient time limits                            analysis/traninit.c:17-38
 */
#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <numeric>

#include "bsim4.h"
#include "dio.h"
#include "circuit.h"

namespace ngsf {

namespace {

const double kBoltz = 1.38064852e-23;
const double kCharge = 1.6021766208e-19;
const double kKoverQ = kBoltz / kCharge;
const double kRefTemp = 27.0 + 273.15;
const double kRoot2 = 1.4142135623730950488016887242097;
const double kCtoK = 273.15;

struct Stamp {
    int row, col;   /* equations; row==-1 marks a right-hand-side stamp */
};

/* one device kind's stamp pattern: for instance i, stamp k */
struct KindStamps {
    int nstamp = 0;                     /* stamps per instance */
    std::vector<std::vector<Stamp>> per;  /* [instance][k] */
};

/* ---------------- MOS1 temperature / model defaults ------------------- */
void mos1_params(const Circuit &c, const Model &m, const Instance &in,
                 double *p /* M1P_COUNT */, bool &needDp, bool &needSp)
{
    const Params &mp = m.p;
    const Options &o = c.opt;
    int type = m.polarity;
    double latDiff = mp.get("ld", 0.0);
    double js = mp.get("js", 0.0);
    double is = mp.get("is", 1e-14);
    bool kpGiven = mp.has("kp");
    double kp = mp.get("kp", 2e-5);
    double cgso = mp.get("cgso", 0.0), cgdo = mp.get("cgdo", 0.0), cgbo = mp.get("cgbo", 0.0);
    bool vt0Given = mp.has("vto") || mp.has("vt0");
    double vt0 = mp.has("vto") ? mp.get("vto", 0.0) : mp.get("vt0", 0.0);
    bool cjGiven = mp.has("cj"), cjswGiven = mp.has("cjsw");
    double cj = mp.get("cj", 0.0), cjsw = mp.get("cjsw", 0.0);
    double pb = mp.get("pb", 0.8), mj = mp.get("mj", 0.5), mjsw = mp.get("mjsw", 0.5);
    double fc = mp.get("fc", 0.5);
    bool phiGiven = mp.has("phi");
    double phi = mp.get("phi", 0.6);
    double lambda = mp.get("lambda", 0.0);
    bool gammaGiven = mp.has("gamma");
    double gamma = mp.get("gamma", 0.0);
    bool rdGiven = mp.has("rd"), rsGiven = mp.has("rs"), rshGiven = mp.has("rsh");
    double rd = mp.get("rd", 0.0), rs = mp.get("rs", 0.0), rsh = mp.get("rsh", 0.0);
    bool cbdGiven = mp.has("cbd"), cbsGiven = mp.has("cbs");
    double cbd = mp.get("cbd", 0.0), cbs = mp.get("cbs", 0.0);
    bool toxGiven = mp.has("tox");
    double tox = mp.get("tox", 0.0);
    bool u0Given = mp.has("u0") || mp.has("uo");
    double u0 = mp.has("u0") ? mp.get("u0", 0.0) : mp.get("uo", 0.0);
    bool nsubGiven = mp.has("nsub");
    double nsub = mp.get("nsub", 0.0);
    bool tpgGiven = mp.has("tpg");
    double tpg = mp.get("tpg", 0.0);
    bool nssGiven = mp.has("nss");
    double nss = mp.get("nss", 0.0);
    double tnom = mp.has("tnom") ? mp.get("tnom", 0.0) + kCtoK : o.tnom;

    /* model part of MOS1temp */
    double fact1 = tnom / kRefTemp;
    double vtnom = tnom * kKoverQ;
    double kt1 = kBoltz * tnom;
    double egfet1 = 1.16 - (7.02e-4 * tnom * tnom) / (tnom + 1108);
    double arg1 = -egfet1 / (kt1 + kt1) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
    double pbfact1 = -2 * vtnom * (1.5 * log(fact1) + kCharge * arg1);
    if (phi <= 0.0)
        throw NetlistError(m.name + ": Phi is not positive.");
    double oxideCapFactor = 0;
    if (!toxGiven || tox == 0) {
        oxideCapFactor = 0;
    } else {
        oxideCapFactor = 3.9 * 8.854214871e-12 / tox;
        if (!kpGiven) {
            if (!u0Given)
                u0 = 600;
            kp = u0 * oxideCapFactor * 1e-4;
        }
        if (nsubGiven) {
            if (nsub * 1e6 > 1.45e16) {
                if (!phiGiven) {
                    phi = 2 * vtnom * log(nsub * 1e6 / 1.45e16);
                    phi = std::max(.1, phi);
                }
                double fermis = type * .5 * phi;
                double wkfng = 3.2;
                if (!tpgGiven)
                    tpg = 1;
                if (tpg != 0) {
                    double fermig = type * tpg * .5 * egfet1;
                    wkfng = 3.25 + .5 * egfet1 - fermig;
                }
                double wkfngs = wkfng - (3.25 + .5 * egfet1 + fermis);
                if (!gammaGiven)
                    gamma = sqrt(2 * 11.70 * 8.854214871e-12 * kCharge * nsub * 1e6) /
                            oxideCapFactor;
                if (!vt0Given) {
                    if (!nssGiven)
                        nss = 0;
                    double vfb = wkfngs - nss * 1e4 * kCharge / oxideCapFactor;
                    vt0 = vfb + type * (gamma * sqrt(phi) + phi);
                }
            } else {
                throw NetlistError(m.name + ": Nsub < Ni");
            }
        }
    }
    (void)js;

    /* instance defaults (MOS1setup / MOS1temp) */
    const Params &ip = in.p;
    double dtemp = ip.get("dtemp", 0.0);
    double temp = ip.has("temp") ? ip.get("temp", 0.0) + kCtoK : o.temp + dtemp;
    double drainArea = ip.get("ad", o.defad), sourceArea = ip.get("as", o.defas);
    double mm = ip.get("m", 1.0);
    double l = ip.get("l", o.defl), w = ip.get("w", o.defw);
    double pd = ip.get("pd", 0.0), ps = ip.get("ps", 0.0);
    double nrd = ip.get("nrd", 1.0), nrs = ip.get("nrs", 1.0);
    double icvds = ip.get("icvds", 0.0), icvgs = ip.get("icvgs", 0.0), icvbs = ip.get("icvbs", 0.0);
    if (ip.vec.count("ic")) {
        const auto &v = ip.vec.at("ic");
        if (v.size() > 0) icvds = v[0];
        if (v.size() > 1) icvgs = v[1];
        if (v.size() > 2) icvbs = v[2];
    }
    needDp = (rd != 0 || (rsh != 0 && nrd != 0));
    needSp = (rs != 0 || (rsh != 0 && nrs != 0));

    double vt = temp * kKoverQ;
    double ratio = temp / tnom;
    double fact2 = temp / kRefTemp;
    double kt = temp * kBoltz;
    double egfet = 1.16 - (7.02e-4 * temp * temp) / (temp + 1108);
    double arg = -egfet / (kt + kt) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
    double pbfact = -2 * vt * (1.5 * log(fact2) + kCharge * arg);
    double ratio4 = ratio * sqrt(ratio);
    double tTransconductance = kp / ratio4;
    double phio = (phi - pbfact1) / fact1;
    double tPhi = fact2 * phio + pbfact;
    double tVbi = vt0 - type * (gamma * sqrt(phi)) + .5 * (egfet1 - egfet) +
                  type * .5 * (tPhi - phi);
    double tVto = tVbi + type * gamma * sqrt(tPhi);
    double tSatCur = is * exp(-egfet / vt + egfet1 / vtnom);
    double tSatCurDens = js * exp(-egfet / vt + egfet1 / vtnom);
    double pbo = (pb - pbfact1) / fact1;
    double gmaold = (pb - pbo) / pbo;
    double capfact = 1 / (1 + mj * (4e-4 * (tnom - kRefTemp) - gmaold));
    double tCbd = cbd * capfact;
    double tCbs = cbs * capfact;
    double tCj = cj * capfact;
    capfact = 1 / (1 + mjsw * (4e-4 * (tnom - kRefTemp) - gmaold));
    double tCjsw = cjsw * capfact;
    double tBulkPot = fact2 * pbo + pbfact;
    double gmanew = (tBulkPot - pbo) / pbo;
    capfact = (1 + mj * (4e-4 * (temp - kRefTemp) - gmanew));
    tCbd *= capfact;
    tCbs *= capfact;
    tCj *= capfact;
    capfact = (1 + mjsw * (4e-4 * (temp - kRefTemp) - gmanew));
    tCjsw *= capfact;
    double tDepCap = fc * tBulkPot;
    double sourceVcrit, drainVcrit;
    if (tSatCurDens == 0 || drainArea == 0 || sourceArea == 0) {
        sourceVcrit = drainVcrit = vt * log(vt / (kRoot2 * mm * tSatCur));
    } else {
        drainVcrit = vt * log(vt / (kRoot2 * mm * tSatCurDens * drainArea));
        sourceVcrit = vt * log(vt / (kRoot2 * mm * tSatCurDens * sourceArea));
    }
    double czbd, czbdsw, czbs, czbssw;
    if (cbdGiven)
        czbd = tCbd * mm;
    else
        czbd = cjGiven ? tCj * mm * drainArea : 0;
    czbdsw = cjswGiven ? tCjsw * pd * mm : 0;
    double a1 = 1 - fc;
    double sarg = exp((-mj) * log(a1));
    double sargsw = exp((-mjsw) * log(a1));
    double f2d = czbd * (1 - fc * (1 + mj)) * sarg / a1 + czbdsw * (1 - fc * (1 + mjsw)) * sargsw / a1;
    double f3d = czbd * mj * sarg / a1 / tBulkPot + czbdsw * mjsw * sargsw / a1 / tBulkPot;
    double f4d = czbd * tBulkPot * (1 - a1 * sarg) / (1 - mj) +
                 czbdsw * tBulkPot * (1 - a1 * sargsw) / (1 - mjsw) -
                 f3d / 2 * (tDepCap * tDepCap) - tDepCap * f2d;
    if (cbsGiven)
        czbs = tCbs * mm;
    else
        czbs = cjGiven ? tCj * sourceArea * mm : 0;
    czbssw = cjswGiven ? tCjsw * ps * mm : 0;
    double f2s = czbs * (1 - fc * (1 + mj)) * sarg / a1 + czbssw * (1 - fc * (1 + mjsw)) * sargsw / a1;
    double f3s = czbs * mj * sarg / a1 / tBulkPot + czbssw * mjsw * sargsw / a1 / tBulkPot;
    double f4s = czbs * tBulkPot * (1 - a1 * sarg) / (1 - mj) +
                 czbssw * tBulkPot * (1 - a1 * sargsw) / (1 - mjsw) -
                 f3s / 2 * (tDepCap * tDepCap) - tDepCap * f2s;
    double gdrain = 0, gsource = 0;
    if (rdGiven)
        gdrain = rd != 0 ? mm / rd : 0;
    else if (rshGiven)
        gdrain = rsh != 0 ? mm / (rsh * nrd) : 0;
    if (rsGiven)
        gsource = rs != 0 ? mm / rs : 0;
    else if (rshGiven)
        gsource = (rsh != 0 && nrs != 0) ? mm / (rsh * nrs) : 0;

    /* load-time constants (mos1load.c:131-154) */
    double Leff = l - 2 * latDiff;
    double DrainSatCur, SourceSatCur;
    if (tSatCurDens == 0 || drainArea == 0 || sourceArea == 0) {
        DrainSatCur = mm * tSatCur;
        SourceSatCur = mm * tSatCur;
    } else {
        DrainSatCur = tSatCurDens * mm * drainArea;
        SourceSatCur = tSatCurDens * mm * sourceArea;
    }
    p[M1P_TYPE] = type;
    p[M1P_VT] = kKoverQ * temp;
    p[M1P_DSAT] = DrainSatCur;
    p[M1P_SSAT] = SourceSatCur;
    p[M1P_CGSO] = cgso * mm * w;
    p[M1P_CGDO] = cgdo * mm * w;
    p[M1P_CGBO] = cgbo * mm * Leff;
    p[M1P_BETA] = tTransconductance * mm * w / Leff;
    p[M1P_COX] = oxideCapFactor * Leff * mm * w;
    p[M1P_TPHI] = tPhi;
    p[M1P_TVBI] = tVbi;
    p[M1P_TVTO] = tVto;
    p[M1P_GAMMA] = gamma;
    p[M1P_LAMBDA] = lambda;
    p[M1P_SVCRIT] = sourceVcrit;
    p[M1P_DVCRIT] = drainVcrit;
    p[M1P_CBS] = czbs;
    p[M1P_CBSSW] = czbssw;
    p[M1P_CBD] = czbd;
    p[M1P_CBDSW] = czbdsw;
    p[M1P_TDEPCAP] = tDepCap;
    p[M1P_TBULKPOT] = tBulkPot;
    p[M1P_F2S] = f2s;
    p[M1P_F3S] = f3s;
    p[M1P_F4S] = f4s;
    p[M1P_F2D] = f2d;
    p[M1P_F3D] = f3d;
    p[M1P_F4D] = f4d;
    p[M1P_MJ] = mj;
    p[M1P_MJSW] = mjsw;
    p[M1P_GDRAIN] = gdrain;
    p[M1P_GSOURCE] = gsource;
    p[M1P_OFF] = ip.has("off") ? 1.0 : 0.0;
    p[M1P_ICVDS] = icvds;
    p[M1P_ICVGS] = icvgs;
    p[M1P_ICVBS] = icvbs;
}

int mk_internal(Circuit &c, const std::string &name, bool voltage)
{
    int id = (int)c.nodeName.size();
    c.nodeName.push_back(name);
    c.nodeIsVoltage.push_back(voltage ? 1 : 0);
    return id;
}

}  // namespace

void compile(Circuit &c, Image &img)
{
    const Options &o = c.opt;
    if (o.method != 0 && o.method != 1)
        throw NetlistError("unknown integration method");
    if (c.uic)
        throw NetlistError(".tran uic is not supported by this engine");
    /* DCtran raises the order only from 1 to 2 (dctran.c:820-830), so the
     * order never exceeds 2 whatever maxord allows (cktsopt.c caps it at
     * 6), and the states past CKTstate3 are never read: the engine keeps
     * four state vectors and runs any maxord >= 2 as 2 */
    if (o.maxord < 1)
        throw NetlistError("maxord must be at least 1");

    /* ---------------- setup: internal nodes, branches, states -------- */
    std::vector<std::array<double, M1P_COUNT>> m1p;
    std::vector<std::array<double, B4P_COUNT>> b4p;
    std::vector<std::array<double, DIP_COUNT>> dip;
    int states = 0;
    for (int kind = 0; kind < K_COUNT; kind++) {
        for (int idx : c.order[kind]) {
            Instance &in = c.inst[idx];
            switch (kind) {
            case K_BSIM4: {
                /* BSIM4setup: state chunk, then internal drain/source nodes
                 * (b4set.c:2317-2530) */
                in.states = states;
                states += B4S_COUNT;
                std::array<double, B4P_COUNT> p{};
                bool needDp, needSp;
                bsim4_params(c, c.models[in.model], in, p.data(), needDp, needSp);
                int d = in.nodes[0], g = in.nodes[1], s = in.nodes[2], b = in.nodes[3];
                int dp = needDp ? mk_internal(c, in.name + "#drain", true) : d;
                int sp = needSp ? mk_internal(c, in.name + "#source", true) : s;
                in.inodes = {d, g, s, b, dp, sp};
                b4p.push_back(p);
                break;
            }
            case K_DIO: {
                /* DIOsetup: states, then the series-resistance node */
                in.states = states;
                states += DIS_COUNT;
                if (in.model < 0)
                    throw NetlistError("diode " + in.name + " needs a model");
                std::array<double, DIP_COUNT> p{};
                bool needPP;
                dio_params(c, c.models[in.model], in, p.data(), needPP);
                int pos = in.nodes[0], neg = in.nodes[1];
                int pp = needPP ? mk_internal(c, in.name + "#internal", true) : pos;
                in.inodes = {pos, neg, pp};
                dip.push_back(p);
                break;
            }
            case K_CAP:
                in.states = states;
                states += 2;
                in.inodes = in.nodes;
                break;
            case K_MOS1: {
                in.states = states;
                states += M1S_COUNT;
                std::array<double, M1P_COUNT> p{};
                bool needDp, needSp;
                mos1_params(c, c.models[in.model], in, p.data(), needDp, needSp);
                int d = in.nodes[0], g = in.nodes[1], s = in.nodes[2], b = in.nodes[3];
                int dp = needDp ? mk_internal(c, in.name + "#drain", true) : d;
                int sp = needSp ? mk_internal(c, in.name + "#source", true) : s;
                in.inodes = {d, g, s, b, dp, sp};
                m1p.push_back(p);
                break;
            }
            case K_VSRC:
                in.branch = mk_internal(c, in.name + "#branch", false);
                in.inodes = {in.nodes[0], in.nodes[1], in.branch};
                break;
            default:
                in.inodes = in.nodes;
                break;
            }
        }
    }
    c.numStates = states;
    const int n = c.n();
    img.n = n;
    img.nstates = states;
    img.names.assign(c.nodeName.begin() + 1, c.nodeName.end());
    img.ntype.assign(c.nodeIsVoltage.begin(), c.nodeIsVoltage.end());

    /* ---------------- per-kind arrays and stamp patterns ------------- */
    int slot = 0;
    struct StampRec { int row, col, slot; };
    std::vector<StampRec> recs;   /* in reference load order */
    auto add_kind = [&](int nk, int nst, const std::function<Stamp(int, int)> &pat) {
        int base = slot;
        for (int i = 0; i < nk; i++)
            for (int k = 0; k < nst; k++) {
                Stamp s = pat(i, k);
                int sl = base + k * nk + i;
                if (s.row < 0) {            /* rhs stamp */
                    if (s.col != 0)
                        recs.push_back({-1, s.col, sl});
                } else if (s.row != 0 && s.col != 0) {
                    recs.push_back({s.row, s.col, sl});
                }
            }
        slot += nk * nst;
        return base;
    };

    /* BSIM4 (kind order: bsim4, cap, dio, isrc, mos1, res, vsrc).  Stamp
     * sequence of BSIM4LoadRhsMat for the supported selectors
     * (b4ld.c:5448-5620): rhs d' g' b' s', then the matrix terms. */
    {
        const auto &ord = c.order[K_BSIM4];
        int nk = (int)ord.size();
        img.nb4 = nk;
        img.b4_node.assign(B4N_COUNT * nk, 0);
        img.b4_st.assign(nk, 0);
        img.b4_p.assign((size_t)B4P_COUNT * nk, 0.0);
        for (int i = 0; i < nk; i++) {
            const Instance &in = c.inst[ord[i]];
            for (int t = 0; t < B4N_COUNT; t++)
                img.b4_node[t * nk + i] = in.inodes[t];
            img.b4_st[i] = in.states;
            for (int t = 0; t < B4P_COUNT; t++)
                img.b4_p[(size_t)t * nk + i] = b4p[i][t];
        }
        img.b4_stamp0 = add_kind(nk, B4_NSTAMP, [&](int i, int k) -> Stamp {
            enum { D = B4N_D, G = B4N_G, S = B4N_S, B = B4N_B, DP = B4N_DP, SP = B4N_SP };
            static const int pat[B4_NSTAMP][2] = {
                {-1, DP}, {-1, G}, {-1, B}, {-1, SP},
                /* GPgp GPdp GPsp GPbp */
                {G, G}, {G, DP}, {G, SP}, {G, B},
                /* DPdp DPd DPgp DPsp DPbp Ddp Dd */
                {DP, DP}, {DP, D}, {DP, G}, {DP, SP}, {DP, B}, {D, DP}, {D, D},
                /* SPdp SPgp SPsp SPs SPbp Ssp Ss */
                {SP, DP}, {SP, G}, {SP, SP}, {SP, S}, {SP, B}, {S, SP}, {S, S},
                /* BPdp BPgp BPsp BPbp */
                {B, DP}, {B, G}, {B, SP}, {B, B},
                /* GIDL: DPdp DPgp DPsp DPbp BPdp BPgp BPsp BPbp */
                {DP, DP}, {DP, G}, {DP, SP}, {DP, B}, {B, DP}, {B, G}, {B, SP}, {B, B},
                /* GISL: SPdp SPgp SPsp SPbp BPdp BPgp BPsp BPbp */
                {SP, DP}, {SP, G}, {SP, SP}, {SP, B}, {B, DP}, {B, G}, {B, SP}, {B, B}};
            int map[B4N_COUNT];
            for (int t = 0; t < B4N_COUNT; t++)
                map[t] = img.b4_node[t * nk + i];
            if (pat[k][0] < 0)
                return {-1, map[pat[k][1]]};
            return {map[pat[k][0]], map[pat[k][1]]};
        });
    }
    /* CAP */
    {
        const auto &ord = c.order[K_CAP];
        int nk = (int)ord.size();
        img.ncap = nk;
        img.cap_node.assign(2 * nk, 0);
        img.cap_st.assign(nk, 0);
        img.cap_c.assign(nk, 0);
        img.cap_m.assign(nk, 1);
        img.cap_ic.assign(nk, 0);
        for (int i = 0; i < nk; i++) {
            const Instance &in = c.inst[ord[i]];
            img.cap_node[i] = in.nodes[0];
            img.cap_node[nk + i] = in.nodes[1];
            img.cap_st[i] = in.states;
            double cval = in.value;
            if (in.model >= 0)
                throw NetlistError("capacitor models are not supported: " + in.name);
            img.cap_c[i] = cval * 1.0 * 1.0;   /* CAPcapac * factor * scale */
            img.cap_m[i] = in.p.get("m", 1.0);
            img.cap_ic[i] = in.p.get("ic", 0.0);
        }
        img.cap_stamp0 = add_kind(nk, 6, [&](int i, int k) -> Stamp {
            int p = img.cap_node[i], q = img.cap_node[nk + i];
            switch (k) {
            case 0: return {p, p};
            case 1: return {q, q};
            case 2: return {p, q};
            case 3: return {q, p};
            case 4: return {-1, p};
            default: return {-1, q};
            }
        });
    }
    /* DIO: DIOload order (dioload.c:785-815) */
    {
        const auto &ord = c.order[K_DIO];
        int nk = (int)ord.size();
        img.ndio = nk;
        img.dio_node.assign(DIN_COUNT * nk, 0);
        img.dio_st.assign(nk, 0);
        img.dio_p.assign((size_t)DIP_COUNT * nk, 0.0);
        for (int i = 0; i < nk; i++) {
            const Instance &in = c.inst[ord[i]];
            for (int t = 0; t < DIN_COUNT; t++)
                img.dio_node[t * nk + i] = in.inodes[t];
            img.dio_st[i] = in.states;
            for (int t = 0; t < DIP_COUNT; t++)
                img.dio_p[(size_t)t * nk + i] = dip[i][t];
        }
        img.dio_stamp0 = add_kind(nk, DIO_NSTAMP, [&](int i, int k) -> Stamp {
            int P = img.dio_node[DIN_POS * nk + i], N = img.dio_node[DIN_NEG * nk + i];
            int PP = img.dio_node[DIN_POSP * nk + i];
            switch (k) {
            case 0: return {-1, N};
            case 1: return {-1, PP};
            case 2: return {P, P};
            case 3: return {N, N};
            case 4: return {PP, PP};
            case 5: return {P, PP};
            case 6: return {N, PP};
            case 7: return {PP, P};
            default: return {PP, N};
            }
        });
    }
    /* ISRC */
    auto fill_src = [&](int kind, std::vector<int> &node, std::vector<int> &wk,
                        std::vector<int> &nc, std::vector<double> &coef,
                        std::vector<double> &dc, std::vector<int> &dcg,
                        std::vector<double> &mv) {
        const auto &ord = c.order[kind];
        int nk = (int)ord.size();
        node.assign(3 * nk, 0);
        wk.assign(nk, 0);
        nc.assign(nk, 0);
        coef.assign((size_t)nk * NGSF_MAX_COEFFS, 0.0);
        dc.assign(nk, 0);
        dcg.assign(nk, 0);
        mv.assign(nk, 1.0);
        for (int i = 0; i < nk; i++) {
            const Instance &in = c.inst[ord[i]];
            /* the current source's instance struct lists its negative node
             * first (isrcdefs.h:30-31), so the first netlist node binds to
             * ISRCnegNode; the voltage source lists the positive node first */
            bool isrc = kind == K_ISRC;
            node[i] = in.nodes[isrc ? 1 : 0];
            node[nk + i] = in.nodes[isrc ? 0 : 1];
            node[2 * nk + i] = in.branch;
            wk[i] = in.wf.kind;
            nc[i] = (int)in.wf.coef.size();
            for (size_t k = 0; k < in.wf.coef.size(); k++)
                coef[(size_t)i * NGSF_MAX_COEFFS + k] = in.wf.coef[k];
            if (in.wf.kind == WF_EXP)
                throw NetlistError("EXP sources are not supported: " + in.name);
            if (in.wf.kind == WF_PULSE && in.wf.coef.size() < 2)
                throw NetlistError("PULSE needs at least V1 V2: " + in.name);
            if (in.wf.kind == WF_SINE && in.wf.coef.size() < 2)
                throw NetlistError("SIN needs at least VO VA: " + in.name);
            if (in.wf.kind == WF_PWL && (in.wf.coef.size() < 2 || in.wf.coef.size() % 2))
                throw NetlistError("PWL needs time/value pairs: " + in.name);
            dc[i] = in.wf.dc;
            dcg[i] = in.wf.dcgiven ? 1 : 0;
            mv[i] = in.p.get("m", 1.0);
        }
        return nk;
    };
    {
        int nk = fill_src(K_ISRC, img.isrc_node, img.isrc_kind, img.isrc_ncoef,
                          img.isrc_coef, img.isrc_dc, img.isrc_dcgiven, img.isrc_m);
        img.nisrc = nk;
        img.isrc_stamp0 = add_kind(nk, 2, [&](int i, int k) -> Stamp {
            return {-1, k == 0 ? img.isrc_node[i] : img.isrc_node[nk + i]};
        });
    }
    /* MOS1 */
    {
        const auto &ord = c.order[K_MOS1];
        int nk = (int)ord.size();
        img.nmos1 = nk;
        img.mos1_node.assign(M1N_COUNT * nk, 0);
        img.mos1_st.assign(nk, 0);
        img.mos1_p.assign((size_t)M1P_COUNT * nk, 0.0);
        for (int i = 0; i < nk; i++) {
            const Instance &in = c.inst[ord[i]];
            for (int t = 0; t < M1N_COUNT; t++)
                img.mos1_node[t * nk + i] = in.inodes[t];
            img.mos1_st[i] = in.states;
            for (int t = 0; t < M1P_COUNT; t++)
                img.mos1_p[(size_t)t * nk + i] = m1p[i][t];
        }
        img.mos1_stamp0 = add_kind(nk, M1_NSTAMP, [&](int i, int k) -> Stamp {
            int d = img.mos1_node[M1N_D * nk + i], g = img.mos1_node[M1N_G * nk + i];
            int s = img.mos1_node[M1N_S * nk + i], b = img.mos1_node[M1N_B * nk + i];
            int dp = img.mos1_node[M1N_DP * nk + i], sp = img.mos1_node[M1N_SP * nk + i];
            static const int pat[M1_NSTAMP][2] = {
                {0, 0}, {1, 1}, {2, 2}, {3, 3}, {4, 4}, {5, 5}, {0, 4}, {1, 3},
                {1, 4}, {1, 5}, {2, 5}, {3, 1}, {3, 4}, {3, 5}, {4, 0}, {4, 1},
                {4, 3}, {4, 5}, {5, 1}, {5, 2}, {5, 3}, {5, 4},
                {-1, 1}, {-1, 3}, {-1, 4}, {-1, 5}};
            int map[6] = {d, g, s, b, dp, sp};
            if (pat[k][0] < 0)
                return {-1, map[pat[k][1]]};
            return {map[pat[k][0]], map[pat[k][1]]};
        });
    }
    /* RES */
    {
        const auto &ord = c.order[K_RES];
        int nk = (int)ord.size();
        img.nres = nk;
        img.res_node.assign(2 * nk, 0);
        img.res_g.assign(nk, 0);
        for (int i = 0; i < nk; i++) {
            const Instance &in = c.inst[ord[i]];
            if (in.model >= 0)
                throw NetlistError("resistor models are not supported: " + in.name);
            img.res_node[i] = in.nodes[0];
            img.res_node[nk + i] = in.nodes[1];
            double r = in.value;
            if (r == 0)
                throw NetlistError("zero-valued resistor: " + in.name);
            double mm = in.p.get("m", 1.0);
            double factor = (((0.0 * 0.0) + 0.0) * 0.0) + 1.0;
            img.res_g[i] = mm / (r * factor * 1.0);
        }
        img.res_stamp0 = add_kind(nk, 4, [&](int i, int k) -> Stamp {
            int p = img.res_node[i], q = img.res_node[nk + i];
            switch (k) {
            case 0: return {p, p};
            case 1: return {q, q};
            case 2: return {p, q};
            default: return {q, p};
            }
        });
    }
    /* VSRC */
    {
        int nk = fill_src(K_VSRC, img.vsrc_node, img.vsrc_kind, img.vsrc_ncoef,
                          img.vsrc_coef, img.vsrc_dc, img.vsrc_dcgiven, img.vsrc_m);
        img.nvsrc = nk;
        img.vsrc_stamp0 = add_kind(nk, 5, [&](int i, int k) -> Stamp {
            int p = img.vsrc_node[i], q = img.vsrc_node[nk + i], br = img.vsrc_node[2 * nk + i];
            switch (k) {
            case 0: return {p, br};
            case 1: return {q, br};
            case 2: return {br, p};
            case 3: return {br, q};
            default: return {-1, br};
            }
        });
    }
    img.nstamp = slot;

    /* ---------------- matrix pattern and gather lists ---------------- */
    /* cells in CSC order (column-major, rows ascending) */
    std::vector<std::pair<int, int>> cells;   /* (col, row), 1-based */
    for (auto &r : recs)
        if (r.row > 0)
            cells.push_back({r.col, r.row});
    std::sort(cells.begin(), cells.end());
    cells.erase(std::unique(cells.begin(), cells.end()), cells.end());
    /* every equation needs at least its column present */
    img.a_cp.assign(n + 1, 0);
    img.a_ri.clear();
    for (auto &cr : cells) {
        img.a_cp[cr.first]++;   /* column cr.first (1-based) -> index cr.first-1 */
        img.a_ri.push_back(cr.second - 1);
    }
    for (int j = 0; j < n; j++)
        img.a_cp[j + 1] += img.a_cp[j];
    int nnz = (int)cells.size();
    auto cell_index = [&](int row, int col) -> int {
        auto it = std::lower_bound(cells.begin(), cells.end(), std::make_pair(col, row));
        return (int)(it - cells.begin());
    };
    std::vector<std::vector<int>> glist(nnz), rlist(n + 1);
    for (auto &r : recs) {
        if (r.row > 0)
            glist[cell_index(r.row, r.col)].push_back(r.slot);
        else
            rlist[r.col].push_back(r.slot);
    }
    img.gptr.assign(nnz + 1, 0);
    img.gsrc.clear();
    for (int p = 0; p < nnz; p++) {
        for (int s : glist[p])
            img.gsrc.push_back(s);
        img.gptr[p + 1] = (int)img.gsrc.size();
    }
    img.rptr.assign(n + 2, 0);
    img.rsrc.clear();
    for (int i = 0; i <= n; i++) {
        if (i > 0)
            for (int s : rlist[i])
                img.rsrc.push_back(s);
        img.rptr[i + 1] = (int)img.rsrc.size();
    }
    img.heavy.clear();
    for (int p = 0; p < nnz; p++)
        if (img.gptr[p + 1] - img.gptr[p] > 64)
            img.heavy.push_back(p);
    for (int r = 0; r <= n; r++)
        if (img.rptr[r + 1] - img.rptr[r] > 64)
            img.heavy.push_back(-r - 1);
    for (int j = 0; j < n; j++)
        if (img.a_cp[j + 1] == img.a_cp[j])
            throw NetlistError("equation " + img.names[j] + " has no matrix entries (floating node)");
    img.a_diag.assign(n, -1);
    for (int j = 0; j < n; j++)
        for (int p = img.a_cp[j]; p < img.a_cp[j + 1]; p++)
            if (img.a_ri[p] == j)
                img.a_diag[j] = p;

    /* ---------------- transient limits (TRANinit) --------------------- */
    ngsf_opts_t &op = img.opt;
    op.reltol = o.reltol;
    op.abstol = o.abstol;
    op.vntol = o.vntol;
    op.chgtol = o.chgtol;
    op.trtol = o.trtol;
    op.gmin = o.gmin;
    op.pivtol = o.pivtol;
    op.pivrel = o.pivrel;
    op.xmu = o.xmu;
    op.temp = o.temp;
    op.itl1 = o.itl1;
    op.itl4 = o.itl4;
    op.maxord = std::min(o.maxord, 2);
    op.method = o.method;
    op.uic = 0;
    op.tstep = c.tstep;
    op.tstop = c.tstop;
    op.tstart = c.tstart;
    double tmax = c.tmaxGiven;
    if (tmax == 0) {
        if (c.tstep < (c.tstop - c.tstart) / 50.0)
            tmax = c.tstep;
        else
            tmax = (c.tstop - c.tstart) / 50.0;
    }
    op.tmax = tmax;
    op.delmin = 1e-11 * tmax;
    op.minbreak = 10.0 * op.delmin;    /* XSPICE variant (dctran.c:160-164) */
}

}  // namespace ngsf
