/*
 * Flat-netlist reader for the transient path.
 *
 * Card semantics follow the reference parser passes (INPpas1 models,
 * INPpas2 instances and dot cards: src/spicelib/parser/inppas1.c,
 * inppas2.c, inp2r.c, inp2c.c, inp2v.c, inp2i.c, inp2d.c, inp2m.c,
 * inp2dot.c, inpdoopt.c).  Numbers are evaluated the way INPevaluate does
 * (src/spicelib/parser/inpeval.c:16-204): digits accumulated into a double
 * mantissa, then scaled by pow(10, exponent), so every parameter value is
 * the same double the reference sees.
 */
#include <algorithm>
#include <cctype>
#include <cmath>
#include <sstream>

#include "circuit.h"

namespace ngsf {

int Circuit::node(const std::string &nm)
{
    std::string k = nm;
    if (k == "gnd")
        k = "0";
    auto it = nodeIndex.find(k);
    if (it != nodeIndex.end())
        return it->second;
    int id = (int)nodeName.size();
    nodeName.push_back(k);
    nodeIsVoltage.push_back(1);
    nodeIndex[k] = id;
    return id;
}

namespace {

/* INPevaluate restated: sign, integer and fraction digits into one double
 * mantissa, optional exponent, one scale-factor letter; value =
 * sign * mantissa * pow(10, exponent). */
bool eval_number(const std::string &tok, double &out)
{
    const char *h = tok.c_str();
    double mantis = 0;
    int expo1 = 0, expo2 = 0, sign = 1, expsgn = 1;
    if (*h == '+')
        h++;
    else if (*h == '-') {
        h++;
        sign = -1;
    }
    if (*h == '\0' || (!isdigit((unsigned char)*h) && *h != '.'))
        return false;
    while (isdigit((unsigned char)*h)) {
        mantis = 10 * mantis + (*h - '0');
        h++;
    }
    if (*h == '\0') {
        out = mantis * sign;
        return true;
    }
    if (*h == '.') {
        h++;
        if (*h == '\0') {
            out = mantis * sign;
            return true;
        }
        while (isdigit((unsigned char)*h)) {
            mantis = 10 * mantis + (*h - '0');
            expo1 -= 1;
            h++;
        }
    }
    if (*h == 'e' || *h == 'd') {
        h++;
        if (*h == '+')
            h++;
        else if (*h == '-') {
            h++;
            expsgn = -1;
        }
        while (isdigit((unsigned char)*h)) {
            expo2 = 10 * expo2 + (*h - '0');
            h++;
        }
    }
    switch (*h) {
    case 't': expo1 += 12; break;
    case 'g': expo1 += 9; break;
    case 'k': expo1 += 3; break;
    case 'u': expo1 -= 6; break;
    case 'n': expo1 -= 9; break;
    case 'p': expo1 -= 12; break;
    case 'f': expo1 -= 15; break;
    case 'a': expo1 -= 18; break;
    case 'm':
        if (h[1] == 'e' && h[2] == 'g')
            expo1 += 6;
        else if (h[1] == 'i' && h[2] == 'l') {
            expo1 -= 6;
            mantis *= 25.4;
        } else
            expo1 -= 3;
        break;
    default: break;
    }
    out = sign * mantis * pow(10.0, (double)(expo1 + expsgn * expo2));
    return true;
}

double number(const std::string &tok, const std::string &ctx)
{
    double v;
    if (!eval_number(tok, v))
        throw NetlistError("bad number '" + tok + "' in: " + ctx);
    return v;
}

/* Split like INPgetTok: whitespace, '=', ',', '(' and ')' separate tokens;
 * '=' is kept as its own token so "w=2u" and "w = 2u" read the same. */
std::vector<std::string> tokenize(const std::string &line)
{
    std::vector<std::string> t;
    std::string cur;
    auto flush = [&] {
        if (!cur.empty()) {
            t.push_back(cur);
            cur.clear();
        }
    };
    for (char ch : line) {
        if (isspace((unsigned char)ch) || ch == ',' || ch == '(' || ch == ')') {
            flush();
        } else if (ch == '=') {
            flush();
            t.push_back("=");
        } else {
            cur.push_back(ch);
        }
    }
    flush();
    return t;
}

/* key=value pairs (a key with no '=' is a flag with value 1) */
void read_params(const std::vector<std::string> &t, size_t i, Params &p,
                 const std::string &ctx)
{
    while (i < t.size()) {
        std::string key = t[i];
        if (i + 1 < t.size() && t[i + 1] == "=") {
            /* vector value: ic=1,2,3 */
            std::vector<double> vals;
            size_t j = i + 2;
            double v;
            while (j < t.size() && eval_number(t[j], v)) {
                vals.push_back(v);
                j++;
            }
            if (vals.empty())
                throw NetlistError("missing value for '" + key + "' in: " + ctx);
            p.v[key] = vals[0];
            if (vals.size() > 1)
                p.vec[key] = vals;
            i = j;
        } else {
            p.v[key] = 1.0;
            i++;
        }
    }
}

const char *kWaveforms[] = {"pulse", "sin", "exp", "pwl"};

void read_source(Circuit &c, Instance &in, const std::vector<std::string> &t,
                 const std::string &ctx)
{
    size_t i = 3;
    double v;
    while (i < t.size()) {
        const std::string &k = t[i];
        if (eval_number(k, v)) {
            in.wf.dc = v;
            in.wf.dcgiven = true;
            i++;
        } else if (k == "dc") {
            if (i + 1 < t.size() && eval_number(t[i + 1], v)) {
                in.wf.dc = v;
                in.wf.dcgiven = true;
                i += 2;
            } else
                throw NetlistError("dc without value: " + ctx);
        } else if (k == "ac") {
            i++;
            int taken = 0;
            while (i < t.size() && taken < 2 && eval_number(t[i], v)) {
                i++;
                taken++;
            }
        } else if (k == "pulse" || k == "sin" || k == "exp" || k == "pwl") {
            in.wf.kind = k == "pulse" ? WF_PULSE : k == "sin" ? WF_SINE
                         : k == "exp" ? WF_EXP : WF_PWL;
            i++;
            in.wf.coef.clear();
            while (i < t.size() && eval_number(t[i], v)) {
                in.wf.coef.push_back(v);
                i++;
            }
            if ((int)in.wf.coef.size() > NGSF_MAX_COEFFS)
                throw NetlistError("too many waveform coefficients: " + ctx);
        } else if (k == "m" && i + 2 < t.size() && t[i + 1] == "=") {
            in.p.v["m"] = number(t[i + 2], ctx);
            i += 3;
        } else {
            throw NetlistError("unsupported source token '" + k + "' in: " + ctx);
        }
    }
    (void)c;
    (void)kWaveforms;
}

int get_model(Circuit &c, const std::string &name, const std::string &ctx)
{
    auto it = c.modelIndex.find(name);
    if (it == c.modelIndex.end())
        throw NetlistError("unknown model '" + name + "' in: " + ctx);
    return it->second;
}

}  // namespace

std::unique_ptr<Circuit> parse_netlist(const std::string &text)
{
    auto c = std::make_unique<Circuit>();
    c->nodeName.push_back("0");
    c->nodeIsVoltage.push_back(1);
    c->nodeIndex["0"] = 0;

    /* ---- card assembly: lower case, continuation, comments -------- */
    std::vector<std::string> cards;
    std::istringstream is(text);
    std::string raw;
    bool first = true, incontrol = false;
    while (std::getline(is, raw)) {
        if (!raw.empty() && raw.back() == '\r')
            raw.pop_back();
        std::string s;
        for (char ch : raw)
            s.push_back((char)tolower((unsigned char)ch));
        if (first) {
            c->title = raw;
            first = false;
            continue;
        }
        size_t b = s.find_first_not_of(" \t");
        if (b == std::string::npos || s[b] == '*')
            continue;
        s = s.substr(b);
        if (incontrol) {
            if (s.compare(0, 5, ".endc") == 0)
                incontrol = false;
            continue;
        }
        if (s.compare(0, 8, ".control") == 0) {
            incontrol = true;
            continue;
        }
        size_t sc = s.find(';');
        if (sc != std::string::npos)
            s = s.substr(0, sc);
        if (s[0] == '+') {
            if (cards.empty())
                throw NetlistError("continuation line without a card");
            cards.back() += " " + s.substr(1);
            continue;
        }
        if (s.compare(0, 4, ".end") == 0 && (s.size() == 4 || isspace((unsigned char)s[4])))
            break;
        cards.push_back(s);
    }

    /* ---- pass 1: models (INPpas1) ----------------------------------- */
    for (const auto &card : cards) {
        if (card.compare(0, 6, ".model") != 0)
            continue;
        auto t = tokenize(card);
        if (t.size() < 3)
            throw NetlistError("short .model card: " + card);
        Model m;
        m.name = t[1];
        const std::string &ty = t[2];
        Params p;
        read_params(t, 3, p, card);
        if (ty == "nmos" || ty == "pmos") {
            m.polarity = ty == "nmos" ? 1 : -1;
            m.level = (int)p.get("level", 1.0);
            if (m.level == 1)
                m.kind = K_MOS1;
            else if (m.level == 14 || m.level == 54)
                m.kind = K_BSIM4;
            else
                throw NetlistError("unsupported MOS level " + std::to_string(m.level) +
                                   " (supported: 1, 14/54): " + card);
        } else if (ty == "d") {
            m.kind = K_DIO;
        } else if (ty == "r") {
            m.kind = K_RES;
        } else if (ty == "c") {
            m.kind = K_CAP;
        } else {
            throw NetlistError("unsupported model type '" + ty + "': " + card);
        }
        m.p = p;
        if (c->modelIndex.count(m.name))
            throw NetlistError("duplicate model " + m.name);
        c->modelIndex[m.name] = -1;          /* created on first use (INPgetMod) */
        c->models.push_back(m);
    }
    /* models are created in the order instances first reference them */
    std::vector<Model> declared = std::move(c->models);
    c->models.clear();
    std::map<std::string, int> declaredIdx;
    for (size_t i = 0; i < declared.size(); i++)
        declaredIdx[declared[i].name] = (int)i;
    c->modelIndex.clear();
    auto use_model = [&](const std::string &name, const std::string &ctx) -> int {
        auto it = c->modelIndex.find(name);
        if (it != c->modelIndex.end())
            return it->second;
        auto d = declaredIdx.find(name);
        if (d == declaredIdx.end())
            throw NetlistError("unknown model '" + name + "' in: " + ctx);
        c->models.push_back(declared[d->second]);
        int id = (int)c->models.size() - 1;
        c->modelIndex[name] = id;
        return id;
    };

    /* ---- pass 2: instances and dot cards (INPpas2) ------------------- */
    for (const auto &card : cards) {
        auto t = tokenize(card);
        if (t.empty())
            continue;
        char k = t[0][0];
        if (k == '.') {
            if (t[0] == ".model")
                continue;
            if (t[0] == ".tran") {
                if (t.size() < 3)
                    throw NetlistError("short .tran: " + card);
                c->haveTran = true;
                c->tstep = number(t[1], card);
                c->tstop = number(t[2], card);
                size_t i = 3;
                double v;
                if (i < t.size() && eval_number(t[i], v)) {
                    c->tstart = v;
                    i++;
                    if (i < t.size() && eval_number(t[i], v)) {
                        c->tmaxGiven = v;
                        i++;
                    }
                }
                for (; i < t.size(); i++)
                    if (t[i] == "uic")
                        c->uic = true;
            } else if (t[0] == ".options" || t[0] == ".option" || t[0] == ".opt") {
                for (size_t i = 1; i < t.size(); i++) {
                    std::string key = t[i];
                    double v = 1.0;
                    if (key == "method" && i + 2 < t.size() && t[i + 1] == "=") {
                        if (t[i + 2] == "gear")
                            c->opt.method = 1;
                        else if (t[i + 2] == "trap" || t[i + 2] == "trapezoidal")
                            c->opt.method = 0;
                        else
                            throw NetlistError("unsupported method: " + card);
                        i += 2;
                        continue;
                    }
                    if (i + 2 < t.size() && t[i + 1] == "=") {
                        v = number(t[i + 2], card);
                        i += 2;
                    }
                    Options &o = c->opt;
                    if (key == "reltol") o.reltol = v;
                    else if (key == "abstol") o.abstol = v;
                    else if (key == "vntol") o.vntol = v;
                    else if (key == "chgtol") o.chgtol = v;
                    else if (key == "trtol") o.trtol = v;
                    else if (key == "gmin") o.gmin = v;
                    else if (key == "pivtol") o.pivtol = v;
                    else if (key == "pivrel") o.pivrel = v;
                    else if (key == "itl1") o.itl1 = (int)v;
                    else if (key == "itl4") o.itl4 = (int)v;
                    else if (key == "maxord") o.maxord = (int)v;
                    else if (key == "temp") o.temp = v + 273.15;
                    else if (key == "tnom") o.tnom = v + 273.15;
                    else if (key == "defl") o.defl = v;
                    else if (key == "defw") o.defw = v;
                    else if (key == "defad") o.defad = v;
                    else if (key == "defas") o.defas = v;
                    else if (key == "klu") o.klu = true;
                    else if (key == "sparse") o.klu = false;
                    else if (key == "trap") o.method = 0;
                    else if (key == "gear") o.method = 1;
                    /* front-end-only options (noacct, ...) are ignored */
                }
            } else if (t[0] == ".ic") {
                for (size_t i = 1; i + 2 < t.size(); i += 3) {
                    if (t[i] != "v" || t[i + 2] != "=")
                        throw NetlistError("unsupported .ic form: " + card);
                }
                throw NetlistError(".ic is not supported by this engine: " + card);
            } else if (t[0] == ".print" || t[0] == ".plot" || t[0] == ".save" ||
                       t[0] == ".probe" || t[0] == ".width" || t[0] == ".meas" ||
                       t[0] == ".title") {
                continue;
            } else {
                throw NetlistError("unsupported dot card: " + card);
            }
            continue;
        }

        Instance in;
        in.name = t[0];
        switch (k) {
        case 'r':
        case 'c': {
            if (t.size() < 3)
                throw NetlistError("short card: " + card);
            in.kind = k == 'r' ? K_RES : K_CAP;
            in.nodes = {c->node(t[1]), c->node(t[2])};
            size_t i = 3;
            double v;
            if (i < t.size() && eval_number(t[i], v)) {
                in.value = v;
                in.valueGiven = true;
                i++;
            } else if (i < t.size() && t[i] != "=" &&
                       (i + 1 >= t.size() || t[i + 1] != "=")) {
                in.model = use_model(t[i], card);
                i++;
            }
            read_params(t, i, in.p, card);
            const char *vk = k == 'r' ? "r" : "c";
            if (!in.valueGiven && in.p.has(vk)) {
                in.value = in.p.get(vk, 0);
                in.valueGiven = true;
            }
            if (!in.valueGiven && k == 'r' && in.p.has("resistance")) {
                in.value = in.p.get("resistance", 0);
                in.valueGiven = true;
            }
            if (!in.valueGiven)
                throw NetlistError("missing value: " + card);
            break;
        }
        case 'v':
        case 'i': {
            if (t.size() < 3)
                throw NetlistError("short card: " + card);
            in.kind = k == 'v' ? K_VSRC : K_ISRC;
            in.nodes = {c->node(t[1]), c->node(t[2])};
            read_source(*c, in, t, card);
            if (k == 'v' && in.nodes[0] == in.nodes[1])
                throw NetlistError("instance " + in.name + " is a shorted VSRC");
            break;
        }
        case 'd': {
            if (t.size() < 4)
                throw NetlistError("short card: " + card);
            in.kind = K_DIO;
            in.nodes = {c->node(t[1]), c->node(t[2])};
            in.model = use_model(t[3], card);
            size_t i = 4;
            double v;
            if (i < t.size() && eval_number(t[i], v)) {
                in.p.v["area"] = v;
                i++;
            }
            read_params(t, i, in.p, card);
            break;
        }
        case 'm': {
            if (t.size() < 6)
                throw NetlistError("short card: " + card);
            in.nodes = {c->node(t[1]), c->node(t[2]), c->node(t[3]), c->node(t[4])};
            in.model = use_model(t[5], card);
            in.kind = c->models[in.model].kind;
            read_params(t, 6, in.p, card);
            break;
        }
        default:
            throw NetlistError("unsupported element '" + t[0] + "'");
        }
        if (in.model >= 0 && c->models[in.model].kind != in.kind)
            throw NetlistError("model kind mismatch: " + card);
        c->inst.push_back(in);
        if (in.model >= 0)
            c->models[in.model].instances.push_back((int)c->inst.size() - 1);
    }
    if (!c->haveTran)
        throw NetlistError("no .tran card");

    /* iteration order per kind: newest model first, newest instance first
     * (CKTmodCrt / CKTcrtElt prepend: analysis/cktmcrt.c:38-39,
     * devices/cktcrte.c:62-64).  Model-less R/C/V/I/D instances belong to
     * a default model created when the first such instance is parsed. */
    int rank = 0;
    std::map<int, int> modelRank;
    std::map<int, std::vector<int>> defaultInst;
    std::map<int, int> defaultModelRank;
    for (size_t i = 0; i < c->inst.size(); i++) {
        const Instance &in = c->inst[i];
        if (in.model >= 0) {
            if (!modelRank.count(in.model))
                modelRank[in.model] = rank++;
        } else {
            if (!defaultModelRank.count(in.kind))
                defaultModelRank[in.kind] = rank++;
            defaultInst[in.kind].push_back((int)i);
        }
    }
    /* BSIM4v7 follows BSIM4 in the device table (devices/dev.c:154-157), so
     * every 4.7 model loads after every 4.8 model */
    const int kV47Last = 1 << 30;
    for (int kk = 0; kk < K_COUNT; kk++) {
        std::vector<std::pair<int, std::vector<int>>> g;
        for (auto &mr : modelRank)
            if (c->models[mr.first].kind == kk)
                g.push_back({mr.second - (c->models[mr.first].bsim4_v47() ? kV47Last : 0),
                             c->models[mr.first].instances});
        if (defaultModelRank.count(kk))
            g.push_back({defaultModelRank[kk], defaultInst[kk]});
        std::sort(g.begin(), g.end(), [](auto &a, auto &b) { return a.first > b.first; });
        for (auto &gr : g)
            for (auto it = gr.second.rbegin(); it != gr.second.rend(); ++it)
                c->order[kk].push_back(*it);
    }
    return c;
}

}  // namespace ngsf
