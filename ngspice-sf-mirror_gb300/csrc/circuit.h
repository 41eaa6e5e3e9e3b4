/*
 * Host-side circuit compiler: flat SPICE netlist -> structure-of-arrays
 * image of one circuit, ready for upload to the GPU transient engine.
 *
 * The compiler mirrors what the reference does between reading a deck and
 * the first CKTload: INPpas1/INPpas2 (cards -> models, instances, nodes),
 * CKTsetup/DEVsetup (internal nodes, branch equations, state slots, matrix
 * elements), CKTtemp/DEVtemperature (temperature-dependent parameters) and
 * SMPpreOrder (symbolic analysis).  It reproduces the reference's equation
 * numbering and device iteration order so that node names, state offsets
 * and the summation order of every matrix cell match.
 */
#ifndef NGSF_CIRCUIT_H
#define NGSF_CIRCUIT_H

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ngsf_types.h"

namespace ngsf {

struct NetlistError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

/* Reference device-table order (src/spicelib/devices/dev.c:142-200),
 * restricted to the types of the transient path. */
enum DevKind { K_BSIM4 = 0, K_CAP, K_DIO, K_ISRC, K_MOS1, K_RES, K_VSRC, K_COUNT };

struct Params {
    std::map<std::string, double> v;
    std::map<std::string, std::vector<double>> vec;
    bool has(const std::string &k) const { return v.count(k) != 0; }
    double get(const std::string &k, double def) const {
        auto it = v.find(k);
        return it == v.end() ? def : it->second;
    }
};

struct Model {
    std::string name;
    DevKind kind;
    int polarity = 1;           /* +1 nmos, -1 pmos */
    int level = 1;
    Params p;
    std::vector<int> instances; /* indices into Circuit::inst, creation order */
    /* A BSIM4 card whose version starts with 4.7 selects the reference's
     * separate BSIM4v7 device (parser/inpdomod.c:297-313); 4.8, "default" or
     * no version select BSIM4 4.8.3. */
    bool bsim4_v47() const {
        if (kind != K_BSIM4 || !p.has("version"))
            return false;
        const double v = p.get("version", 4.8);
        return v >= 4.7 - 1e-9 && v < 4.8 - 1e-9;
    }
};

struct Waveform {
    int kind = WF_DC;
    std::vector<double> coef;
    double dc = 0.0;
    bool dcgiven = false;
};

struct Instance {
    std::string name;
    DevKind kind;
    std::vector<int> nodes;     /* external terminals, equation numbers */
    int model = -1;             /* index into Circuit::models (or -1) */
    Params p;
    Waveform wf;                /* sources */
    double value = 0.0;         /* R / C value */
    bool valueGiven = false;
    /* filled by setup */
    std::vector<int> inodes;    /* terminals incl. internal nodes */
    int states = 0;             /* state offset */
    int branch = 0;             /* branch equation (vsrc) */
};

struct Options {
    double reltol = 1e-3, abstol = 1e-12, vntol = 1e-6, chgtol = 1e-14;
    double trtol = 7.0, gmin = 1e-12, pivtol = 1e-13, pivrel = 1e-3;
    double xmu = 0.5, temp = 300.15, tnom = 300.15;
    double defl = 1e-4, defw = 1e-4, defad = 0.0, defas = 0.0;
    int itl1 = 100, itl4 = 10, maxord = 2, method = 0; /* 0 trap, 1 gear */
    bool klu = false;
};

struct Circuit {
    std::string title;
    std::vector<std::string> nodeName;   /* [0] = ground */
    std::vector<int> nodeIsVoltage;      /* 1 voltage node, 0 branch current */
    std::map<std::string, int> nodeIndex;
    std::vector<Model> models;
    std::map<std::string, int> modelIndex;
    std::vector<Instance> inst;
    Options opt;
    bool haveTran = false;
    double tstep = 0, tstop = 0, tstart = 0, tmaxGiven = 0;
    bool uic = false;
    std::vector<std::pair<std::string, double>> ics;

    int numStates = 0;
    /* instances per device kind in the reference iteration order
     * (model list newest first, instance list newest first) */
    std::vector<int> order[K_COUNT];

    int n() const { return (int)nodeName.size() - 1; }
    int node(const std::string &nm);     /* find or create */
};

/* Parse a flat netlist.  Throws NetlistError on anything unsupported. */
std::unique_ptr<Circuit> parse_netlist(const std::string &text);

/* Host image of a compiled circuit: plain arrays, sizes and offsets,
 * uploaded verbatim by the engine. */
struct Image {
    int n = 0, nstates = 0, nstamp = 0, nlu = 0;
    ngsf_opts_t opt{};
    /* devices */
    int nb4 = 0;
    std::vector<int> b4_node, b4_st;
    std::vector<double> b4_p;
    int b4_stamp0 = 0;
    int nmos1 = 0, ndio = 0, nres = 0, ncap = 0, nvsrc = 0, nisrc = 0;
    std::vector<int> mos1_node, mos1_st;
    std::vector<double> mos1_p;
    int mos1_stamp0 = 0;
    std::vector<int> dio_node, dio_st;
    std::vector<double> dio_p;
    int dio_stamp0 = 0;
    std::vector<int> res_node;
    std::vector<double> res_g;
    int res_stamp0 = 0;
    std::vector<int> cap_node, cap_st;
    std::vector<double> cap_c, cap_m, cap_ic;
    int cap_stamp0 = 0;
    std::vector<int> vsrc_node, vsrc_kind, vsrc_ncoef, vsrc_dcgiven;
    std::vector<double> vsrc_coef, vsrc_dc, vsrc_m;
    int vsrc_stamp0 = 0;
    std::vector<int> isrc_node, isrc_kind, isrc_ncoef, isrc_dcgiven;
    std::vector<double> isrc_coef, isrc_dc, isrc_m;
    int isrc_stamp0 = 0;
    std::vector<int> ntype;
    /* stamping */
    std::vector<int> gptr, gsrc, rptr, rsrc;
    std::vector<int> heavy;   /* entries with more than 64 terms (rhs row r as -r-1) */
    /* A pattern: CSC over columns 0..n-1 (equation j+1), 0-based rows */
    std::vector<int> a_cp, a_ri, a_lupos, a_diag;
    /* LU */
    std::vector<int> lvl_ptr, lvl_col, cdiag, cend, cbeg, kptr, kdep, kpos, kseg;
    std::vector<int> upd_dst, upd_src, prow, pcol;
    std::vector<int> fl_ptr, fl_row, bl_ptr, bl_row;
    std::vector<int> lr_ptr, lr_col, lr_pos, ur_ptr, ur_col, ur_pos;
    std::vector<int> fh_ptr, fh_row, bh_ptr, bh_row;   /* solve rows reduced by a warp */
    /* right-looking level schedule (large matrices) */
    std::vector<int> rl_ptr, rl_col, sc_ptr, sc_pos, sc_piv;
    std::vector<int> ud_ptr, ud_dst, ud_cptr, ud_l, ud_u, ud_p;
    double lu_flops = 0;   /* multiply-adds of one refactorization */
    int btf_blocks = 0;    /* diagonal blocks of the KLU order (NGSF_ORDER=klu) */
    std::vector<std::string> names;  /* equation names 1..n */
};

/* BSIM4 instance resolution (bsim4_setup.cpp): fills B4P_COUNT values. */
void bsim4_params(const Circuit &c, const Model &m, const Instance &in, double *p,
                  bool &needDp, bool &needSp);

/* Junction diode resolution (dio_setup.cpp): fills DIP_COUNT values. */
void dio_params(const Circuit &c, const Model &m, const Instance &in, double *p,
                bool &needPosPrime);

/* CKTsetup + CKTtemp + SMPpreOrder equivalent. */
void compile(Circuit &c, Image &img);

}  // namespace ngsf

#endif
