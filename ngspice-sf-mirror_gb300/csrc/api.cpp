/*
 * C ABI: engine entry points (include/ngspice_gb300.h) and the
 * sharedspice-compatible API (include/sharedspice.h).
 *
 * The sharedspice layer keeps the reference's observable behaviour for the
 * transient path (src/sharedspice.c): commands are executed immediately,
 * "bg_run" runs the analysis on a background thread and reports through
 * BGThreadRunning ("bg_halt" stops it between windows, "bg_resume"
 * continues it), every accepted point is sent through SendData as the
 * run's windows end, after
 * SendInitData has described the vectors, output vectors are looked up by
 * name with ngGet_Vec_Info, errors return 1.
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ngspice_gb300.h"
#include "../../include/sharedspice.h"
#include "bsim4.h"
#include "circuit.h"
#include "dio.h"
#include "runtime.h"
#include "sparse.h"

using namespace ngsf;

struct ngsf_handle {
    Prepared p;
};

namespace {
thread_local std::string g_err;
thread_local int g_launches = 0;
}  // namespace

/* internal (not exported): engine.cu entry points reach a handle's device
 * descriptor and report errors through ngsf_last_error() */
extern "C" const ngsf_ckt_t *ngsf_internal_desc(const ngsf_handle *h)
{
    return (h && h->p.dev) ? &h->p.dev->desc() : nullptr;
}
extern "C" void ngsf_internal_set_error(const char *msg) { g_err = msg ? msg : ""; }
extern "C" const ngsf_ckt_t *ngsf_internal_ddesc(const ngsf_handle *h)
{
    return (h && h->p.dev) ? h->p.dev->device_desc() : nullptr;
}
extern "C" int ngsf_internal_lufac(ngsf_handle *h, double diag_gmin);

namespace {

int fail(const std::string &msg, int code = -1)
{
    g_err = msg;
    return code;
}

/* probe names: whitespace separated, matched in lower case */
std::vector<std::string> probe_names(const char *probes)
{
    std::vector<std::string> pr;
    if (probes) {
        std::istringstream is(probes);
        std::string t;
        while (is >> t) {
            for (auto &ch : t)
                ch = (char)tolower((unsigned char)ch);
            pr.push_back(t);
        }
    }
    return pr;
}
}  // namespace

extern "C" {

NGSF_API const char *ngsf_last_error(void) { return g_err.c_str(); }

NGSF_API ngsf_handle *ngsf_open(const char *netlist, const char *probes, int outcap, int capmax)
{
    try {
        auto h = std::make_unique<ngsf_handle>();
        prepare(h->p, netlist ? netlist : "", probe_names(probes), outcap > 0 ? outcap : 1,
                capmax > 0 ? capmax : 0);
        return h.release();
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

NGSF_API int ngsf_open_many(const char *const *netlists, int count, const char *probes,
                            int outcap, int capmax, ngsf_handle **out)
{
    if (count < 0 || (count > 0 && (!netlists || !out)))
        return fail("ngsf_open_many: bad arguments");
    try {
        const std::vector<std::string> pr = probe_names(probes);
        std::vector<std::unique_ptr<ngsf_handle>> hs(count);
        std::vector<std::string> errs(count);
        /* parse and compile on all host cores; each netlist only touches
         * its own circuit */
        std::atomic<int> cursor{0};
        auto work = [&]() {
            for (int i; (i = cursor.fetch_add(1)) < count;) {
                try {
                    hs[i] = std::make_unique<ngsf_handle>();
                    prepare_host(hs[i]->p, netlists[i] ? netlists[i] : "", pr);
                } catch (const std::exception &e) {
                    errs[i] = e.what();
                }
            }
        };
        unsigned nt = std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()),
                                         (unsigned)std::max(1, count));
        std::vector<std::thread> pool;
        try {
            /* room for every thread first: emplace_back then never
             * reallocates while started threads are joinable */
            pool.reserve(nt);
            for (unsigned k = 1; k < nt; k++)
                pool.emplace_back(work);
        } catch (...) {
            /* fewer threads: the calling thread takes the rest */
        }
        work();
        for (auto &th : pool)
            th.join();
        for (int i = 0; i < count; i++)
            if (!errs[i].empty())
                return fail("netlist " + std::to_string(i) + ": " + errs[i]);
        /* device allocation and upload on the calling thread (its device) */
        for (int i = 0; i < count; i++)
            prepare_device(hs[i]->p, outcap > 0 ? outcap : 1, capmax > 0 ? capmax : 0);
        for (int i = 0; i < count; i++)
            out[i] = hs[i].release();
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

NGSF_API ngsf_handle *ngsf_compile(const char *netlist)
{
    try {
        auto h = std::make_unique<ngsf_handle>();
        h->p.ckt = parse_netlist(netlist ? netlist : "");
        compile(*h->p.ckt, h->p.img);
        return h.release();
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

NGSF_API void ngsf_close(ngsf_handle *h) { delete h; }

NGSF_API int ngsf_info(const ngsf_handle *h, int *n, int *nnz, int *nstates, int *nlu)
{
    if (!h)
        return fail("null handle");
    if (n) *n = h->p.img.n;
    if (nnz) *nnz = (int)h->p.img.a_ri.size();
    if (nstates) *nstates = h->p.img.nstates;
    if (nlu) *nlu = h->p.img.nlu;
    return 0;
}

NGSF_API int ngsf_eq_name(const ngsf_handle *h, int eq, char *buf, int len)
{
    if (!h || eq < 1 || eq > h->p.img.n || !buf || len <= 0)
        return fail("bad equation");
    snprintf(buf, (size_t)len, "%s", h->p.img.names[eq - 1].c_str());
    return 0;
}

NGSF_API int ngsf_pattern(const ngsf_handle *h, int *colptr, int *rowidx)
{
    if (!h)
        return fail("null handle");
    const Image &m = h->p.img;
    if (colptr)
        memcpy(colptr, m.a_cp.data(), m.a_cp.size() * sizeof(int));
    if (rowidx)
        memcpy(rowidx, m.a_ri.data(), m.a_ri.size() * sizeof(int));
    return 0;
}

NGSF_API int ngsf_probes(const ngsf_handle *h, int *eqs, int max)
{
    if (!h)
        return fail("null handle");
    int n = (int)h->p.probes.size();
    for (int i = 0; i < n && i < max; i++)
        eqs[i] = h->p.probes[i];
    return n;
}

NGSF_API int ngsf_run(ngsf_handle *const *hs, int count, long long max_steps, double *seconds)
{
    try {
        std::vector<Prepared *> cs;
        for (int i = 0; i < count; i++) {
            if (!hs[i])
                return fail("null handle");
            if (!hs[i]->p.dev)
                return fail("circuit was compiled without a device (ngsf_compile)");
            cs.push_back(&hs[i]->p);
        }
        run_batch(cs, max_steps > 0 ? max_steps : 100000000LL, seconds, &g_launches);
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

NGSF_API int ngsf_run_window(ngsf_handle *const *hs, int count, double t_until,
                            long long max_steps, double *seconds)
{
    try {
        std::vector<Prepared *> cs;
        for (int i = 0; i < count; i++) {
            if (!hs[i])
                return fail("null handle");
            if (!hs[i]->p.dev)
                return fail("circuit was compiled without a device (ngsf_compile)");
            cs.push_back(&hs[i]->p);
        }
        run_batch(cs, max_steps > 0 ? max_steps : 100000000LL, seconds, &g_launches, t_until,
                  true);
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

NGSF_API int ngsf_results(const ngsf_handle *h, int *ires, double *fres)
{
    if (!h || h->p.ires.empty())
        return fail("no results");
    if (ires)
        memcpy(ires, h->p.ires.data(), NGSF_R_COUNT * sizeof(int));
    if (fres)
        memcpy(fres, h->p.fres.data(), NGSF_F_COUNT * sizeof(double));
    return 0;
}

NGSF_API int ngsf_points(const ngsf_handle *h, double *buf, int maxpoints)
{
    if (!h)
        return fail("null handle");
    int w = 1 + (int)h->p.probes.size();
    int np = (int)(h->p.points.size() / (size_t)w);
    if (np > maxpoints)
        np = maxpoints;
    if (buf && np)
        memcpy(buf, h->p.points.data(), (size_t)np * w * sizeof(double));
    return np;
}

NGSF_API int ngsf_capture(ngsf_handle *h, double *ax, double *rhs, double *rhsold, double *meta,
                          int maxcap)
{
    try {
        if (!h || h->p.ires.empty())
            return fail("no results");
        int nc = h->p.ires[NGSF_R_NCAP];
        std::vector<double> a, r, m;
        h->p.dev->read_capture(nc, a, r, m);
        int n1 = h->p.img.n + 1;
        int nnz = (int)h->p.img.a_ri.size();
        int capmax = (int)(r.size() / (2 * (size_t)n1));
        int k = nc < maxcap ? nc : maxcap;
        if (k > capmax)
            k = capmax;
        for (int c = 0; c < k; c++) {
            if (ax)
                memcpy(ax + (size_t)c * nnz, a.data() + (size_t)c * nnz, nnz * sizeof(double));
            if (rhs)
                memcpy(rhs + (size_t)c * n1, r.data() + (size_t)c * n1, n1 * sizeof(double));
            if (rhsold)
                memcpy(rhsold + (size_t)c * n1, r.data() + (size_t)(capmax + c) * n1,
                       n1 * sizeof(double));
            if (meta)
                memcpy(meta + 4 * c, m.data() + 4 * c, 4 * sizeof(double));
        }
        return k;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

NGSF_API double ngsf_lu_flops(const ngsf_handle *h) { return h ? h->p.img.lu_flops : 0.0; }

NGSF_API int ngsf_last_launches(void) { return g_launches; }

NGSF_API int ngsf_workload(const ngsf_handle *h, long long *counts)
{
    if (!h)
        return fail("null handle");
    const Image &m = h->p.img;
    counts[0] = m.nmos1;
    counts[1] = m.nres;
    counts[2] = m.ncap;
    counts[3] = m.nvsrc;
    counts[4] = m.nisrc;
    counts[5] = (long long)m.a_ri.size();
    counts[6] = m.nlu;
    counts[7] = m.n;
    counts[8] = m.nb4;
    counts[9] = m.ndio;
    return 0;
}

NGSF_API long long ngsf_device_bytes(const ngsf_handle *h)
{
    return (h && h->p.dev) ? (long long)h->p.dev->bytes() : 0;
}

NGSF_API int ngsf_node_graph(const ngsf_handle *h, int *nv, int *nedges, int *vnode, int *gptr,
                             int *gidx, float *stat)
{
    if (!h)
        return fail("null handle");
    ngsf::PredGraph g = ngsf::pred_graph(h->p.img);
    if (nv)
        *nv = (int)g.vnode.size();
    if (nedges)
        *nedges = (int)g.gidx.size();
    if (vnode)
        memcpy(vnode, g.vnode.data(), g.vnode.size() * sizeof(int));
    if (gptr)
        memcpy(gptr, g.gptr.data(), g.gptr.size() * sizeof(int));
    if (gidx)
        memcpy(gidx, g.gidx.data(), g.gidx.size() * sizeof(int));
    if (stat)
        memcpy(stat, g.stat.data(), g.stat.size() * sizeof(float));
    return 0;
}

NGSF_API int ngsf_wide_info(const ngsf_handle *h, int *wide, int *blocks)
{
    if (!h || !h->p.dev)
        return fail("ngsf_wide_info: null or host-only handle");
    if (wide)
        *wide = h->p.wide ? 1 : 0;
    if (blocks)
        *blocks = h->p.wide_blocks;
    return 0;
}

NGSF_API int ngsf_set_factor_shape(ngsf_handle *h, int blocks, int small_work)
{
    if (!h || !h->p.dev)
        return fail("ngsf_set_factor_shape: null or host-only handle");
    if (blocks < 0 || small_work < 0)
        return fail("ngsf_set_factor_shape: negative shape");
    try {
        h->p.dev->set_factor_shape(blocks, small_work);
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

NGSF_API int ngsf_set_predictor(ngsf_handle *h, int kind, const float *params)
{
    if (!h || !h->p.dev)
        return fail("ngsf_set_predictor: null or host-only handle");
    if (kind < 0 || kind > 3 || (kind == 2 && !params))
        return fail("ngsf_set_predictor: kind 0, 1, 3, or 2 with parameters");
    try {
        h->p.dev->set_pred(h->p.img, kind, params);
    } catch (const std::exception &e) {
        return fail(e.what());
    }
    return 0;
}

NGSF_API int ngsf_set_sync(ngsf_handle *h, int on)
{
    if (!h || !h->p.dev)
        return fail("ngsf_set_sync: null or host-only handle");
    try {
        h->p.dev->set_sync(on != 0);
    } catch (const std::exception &e) {
        return fail(e.what());
    }
    return 0;
}

NGSF_API int ngsf_sync_point(const ngsf_handle *h, int *loc, int *redostep, double *time,
                             double *delta, double *olddelta)
{
    if (!h || h->p.ires.size() < NGSF_R_ALL || h->p.fres.size() < NGSF_F_ALL)
        return 0;
    const int at = h->p.ires[NGSF_R_SYNCLOC];
    if (h->p.ires[NGSF_R_STATUS] != NGSF_HELD || at == 0)
        return 0;
    if (loc)
        *loc = at - 1;
    if (redostep)
        *redostep = h->p.ires[NGSF_R_SYNCREDO];
    if (time)
        *time = h->p.fres[NGSF_F_TIME];
    if (delta)
        *delta = h->p.fres[NGSF_F_DELTA];
    if (olddelta)
        *olddelta = at == 1 ? 0.0 : h->p.fres[NGSF_F_OLDDELTA];
    return 1;
}

NGSF_API int ngsf_sync_reply(ngsf_handle *h, double delta, int redo)
{
    if (!ngsf_sync_point(h, nullptr, nullptr, nullptr, nullptr, nullptr))
        return fail("ngsf_sync_reply: the circuit is not stopped at a sync point");
    if (!(delta > 0.0) || !std::isfinite(delta))
        return fail("ngsf_sync_reply: delta must be positive and finite");
    try {
        h->p.dev->sync_reply(delta, redo ? 1 : 0);
    } catch (const std::exception &e) {
        return fail(e.what());
    }
    return 0;
}

}  // extern "C"

/* ====================================================================== */
/* sharedspice layer                                                       */
/* ====================================================================== */
namespace {

struct Vec {
    std::string name;
    std::vector<double> data;
    vector_info info{};
};

struct Plot {
    std::string name, title, type;
    std::vector<std::unique_ptr<Vec>> vecs;
};

struct Shared {
    std::recursive_mutex mu;
    SendChar *pfcn = nullptr;
    SendStat *statfcn = nullptr;
    ControlledExit *ngexit = nullptr;
    SendData *datfcn = nullptr;
    SendInitData *initfcn = nullptr;
    BGThreadRunning *bgfcn = nullptr;
    GetSyncData *syncfcn = nullptr;
    void *user = nullptr;
    int ident = 0;
    std::string deck;                 /* current circuit text */
    std::vector<std::unique_ptr<Plot>> plots;
    int cur = -1;
    std::thread bg;
    bool running = false;
    std::vector<char *> nameList;     /* storage for AllPlots/AllVecs */
    std::vector<std::string> nameStore;
    std::vector<double> extraBreaks;
    int tranCount = 0;
    /* the transient in progress: run window by window so that accepted
     * points stream out through SendData and bg_halt can stop it between
     * windows (bg_resume continues it) */
    ngsf_handle *active = nullptr;
    Plot *activePlot = nullptr;
    int activeWindow = 0;
    size_t activeSent = 0;
    std::atomic<bool> haltReq{false};
} S;

/* windows a transient is cut into for streaming (each 1/64 of tstop) */
constexpr int kStreamWindows = 64;

void say(const char *fmt, ...)
{
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (S.pfcn)
        S.pfcn(buf, S.ident, S.user);
}

std::string lower(std::string s)
{
    for (auto &c : s)
        c = (char)tolower((unsigned char)c);
    return s;
}

/* replace (or add) the .tran card of the deck */
std::string with_tran(const std::string &deck, const std::string &tranArgs)
{
    std::istringstream is(deck);
    std::ostringstream os;
    std::string line;
    bool first = true;
    while (std::getline(is, line)) {
        std::string l = lower(line);
        size_t b = l.find_first_not_of(" \t");
        if (!first && b != std::string::npos && l.compare(b, 5, ".tran") == 0)
            continue;
        if (!first && b != std::string::npos && l.compare(b, 4, ".end") == 0 &&
            (l.size() == b + 4 || isspace((unsigned char)l[b + 4]))) {
            if (!tranArgs.empty())
                os << ".tran " << tranArgs << "\n";
            os << line << "\n";
            first = false;
            continue;
        }
        os << line << "\n";
        first = false;
    }
    return os.str();
}

/* point the vectors' info at their storage (after appends) */
void refresh_infos(Plot *plot)
{
    for (auto &v : plot->vecs) {
        v->info.v_realdata = v->data.data();
        v->info.v_length = (int)v->data.size();
    }
}

void finish_tran(int status)
{
    ngsf_close(S.active);
    S.active = nullptr;
    S.activePlot = nullptr;
    if (S.statfcn) {
        char st[] = "--ready--";
        S.statfcn(st, S.ident, S.user);
    }
    (void)status;
}

/* Run the active transient window by window until it ends or a halt is
 * requested: after each window the new accepted points are appended to
 * the plot's vectors and sent through SendData (the reference sends each
 * accepted point from CKTdump as it is computed, src/spicelib/analysis/
 * cktdump.c:33 -> OUTpData; here they come one window at a time).
 * Returns 0, or 1 on an error; *halted tells a halt apart from the end. */
int continue_tran(bool *halted)
{
    *halted = false;
    ngsf_handle *h = S.active;
    Plot *plot = S.activePlot;
    const double tstop = h->p.img.opt.tstop;
    const int n = h->p.img.n;
    const int w = 1 + (int)h->p.probes.size();
    size_t nv = plot->vecs.size();
    std::vector<vecvalues> vv(nv);
    std::vector<pvecvalues> pv(nv);
    for (size_t i = 0; i < nv; i++) {
        vv[i].name = (char *)plot->vecs[i]->name.c_str();
        vv[i].cimag = 0;
        vv[i].is_scale = i == 0;
        vv[i].is_complex = false;
        pv[i] = &vv[i];
    }
    const double delmin = h->p.img.opt.delmin;
    while (S.activeWindow < kStreamWindows) {
        const int k = S.activeWindow;
        const double until = k + 1 == kStreamWindows ? 2 * tstop : tstop * (k + 1) / kStreamWindows;
        if (ngsf_run_window(&h, 1, until, 0, nullptr)) {
            say("stderr Error: %s", ngsf_last_error());
            finish_tran(1);
            return 1;
        }
        int ires[NGSF_R_COUNT];
        ngsf_results(h, ires, nullptr);
        const int status = ires[NGSF_R_STATUS];
        const std::vector<double> &pts = h->p.points;
        const size_t np = std::min<size_t>((size_t)ires[NGSF_R_NPOINTS], pts.size() / w);
        const size_t from = S.activeSent;
        {
            std::lock_guard<std::recursive_mutex> g(S.mu);
            for (size_t q = from; q < np; q++) {
                plot->vecs[0]->data.push_back(pts[q * w]);
                for (int i = 0; i < n; i++)
                    plot->vecs[1 + i]->data.push_back(pts[q * w + 1 + i]);
            }
            refresh_infos(plot);
        }
        S.activeSent = np;
        if (S.datfcn)
            for (size_t q = from; q < np; q++) {
                for (size_t i = 0; i < nv; i++)
                    vv[i].creal = plot->vecs[i]->data[q];
                vecvaluesall all{(int)nv, (int)q, pv.data()};
                S.datfcn(&all, (int)nv, S.ident, S.user);
            }
        if (S.statfcn && np) {
            char st[64];
            snprintf(st, sizeof st, "tran %.1f%%", 100.0 * pts[(np - 1) * w] / tstop);
            S.statfcn(st, S.ident, S.user);
        }
        if (status == 0) {
            finish_tran(0);
            return 0;
        }
        if (status != NGSF_HELD) {
            say("stderr Error: transient analysis failed with code %d (time %g)", status,
                h->p.fres[NGSF_F_TIME]);
            finish_tran(1);
            return 1;
        }
        int loc = 0, redo = 0;
        double time = 0, delta = 0, olddelta = 0;
        const bool atSync = ngsf_sync_point(h, &loc, &redo, &time, &delta, &olddelta) != 0;
        if (atSync) {
            /* sharedsync (sharedspice.c:2437-2490): the caller may change
             * delta and ask for the step again; delta stays short of the
             * final time */
            int ret = 0;
            if (S.syncfcn)
                ret = S.syncfcn(time, &delta, olddelta, redo, S.ident, loc, S.user);
            if (redo) {
                if (time + delta > tstop)
                    delta = tstop - time - 1.1 * delmin;
            } else if (time + delta > tstop) {
                double nd = tstop - time - 1.1 * delmin;
                if (nd <= 0.0)
                    nd = tstop - time;
                delta = nd;
            }
            if (ngsf_sync_reply(h, delta, ret)) {
                say("stderr Error: %s", ngsf_last_error());
                finish_tran(1);
                return 1;
            }
        } else {
            S.activeWindow++;
        }
        if (S.haltReq.load()) {
            *halted = true;
            return 0;
        }
    }
    finish_tran(0);
    return 0;
}

int do_tran(const std::string &tranArgs)
{
    std::string deck;
    {
        std::lock_guard<std::recursive_mutex> g(S.mu);
        if (S.deck.empty()) {
            say("stderr Error: there is no circuit loaded");
            return 1;
        }
        deck = tranArgs.empty() ? S.deck : with_tran(S.deck, tranArgs);
    }
    if (S.active) {
        ngsf_close(S.active);
        S.active = nullptr;
    }
    ngsf_handle *h = ngsf_open(deck.c_str(), nullptr, 1 << 22, 0);
    if (!h) {
        say("stderr Error: %s", ngsf_last_error());
        return 1;
    }
    if (S.statfcn) {
        char st[] = "tran 0.0%";
        S.statfcn(st, S.ident, S.user);
    }
    auto plot = std::make_unique<Plot>();
    plot->name = "tran" + std::to_string(++S.tranCount);
    plot->title = h->p.ckt->title;
    plot->type = "transient";
    int n = h->p.img.n;
    auto tv = std::make_unique<Vec>();
    tv->name = "time";
    plot->vecs.push_back(std::move(tv));
    for (int i = 0; i < n; i++) {
        auto v = std::make_unique<Vec>();
        v->name = h->p.img.names[i];
        plot->vecs.push_back(std::move(v));
    }
    for (auto &v : plot->vecs) {
        v->info.v_name = (char *)v->name.c_str();
        v->info.v_type = v->name == "time" ? 1 : (v->name.find("#branch") != std::string::npos ? 4 : 3);
        v->info.v_flags = 1;   /* VF_REAL */
        v->info.v_compdata = nullptr;
    }
    refresh_infos(plot.get());
    /* SendInitData once, then SendData per accepted point as windows end */
    if (S.initfcn) {
        std::vector<vecinfo> vi(plot->vecs.size());
        std::vector<pvecinfo> pvi(plot->vecs.size());
        for (size_t i = 0; i < plot->vecs.size(); i++) {
            vi[i].number = (int)i;
            vi[i].vecname = (char *)plot->vecs[i]->name.c_str();
            vi[i].is_real = true;
            vi[i].pdvec = &plot->vecs[i]->info;
            vi[i].pdvecscale = &plot->vecs[0]->info;
            pvi[i] = &vi[i];
        }
        vecinfoall all{(char *)plot->name.c_str(), (char *)plot->title.c_str(),
                       (char *)"", (char *)plot->type.c_str(), (int)vi.size(), pvi.data()};
        S.initfcn(&all, S.ident, S.user);
    }
    {
        std::lock_guard<std::recursive_mutex> g(S.mu);
        S.activePlot = plot.get();
        S.plots.push_back(std::move(plot));
        S.cur = (int)S.plots.size() - 1;
    }
    if (S.syncfcn && ngsf_set_sync(h, 1)) {
        say("stderr Error: %s", ngsf_last_error());
        ngsf_close(h);
        return 1;
    }
    S.active = h;
    S.activeWindow = 0;
    S.activeSent = 0;
    S.haltReq = false;
    bool halted = false;
    return continue_tran(&halted);
}

/* bg_run / bg_resume: the transient on the background thread */
void start_bg(std::function<void()> body)
{
    if (S.bg.joinable())
        S.bg.join();
    S.running = true;
    if (S.bgfcn)
        S.bgfcn(false, S.ident, S.user);
    S.bg = std::thread([body] {
        body();
        S.running = false;
        if (S.bgfcn)
            S.bgfcn(true, S.ident, S.user);
    });
}

std::string g_lastTran;

int command(const std::string &raw)
{
    std::string cmd = raw;
    size_t b = cmd.find_first_not_of(" \t");
    if (b == std::string::npos)
        return 0;
    cmd = cmd.substr(b);
    std::istringstream is(cmd);
    std::string verb;
    is >> verb;
    verb = lower(verb);
    std::string rest;
    std::getline(is, rest);
    if (verb == "source") {
        std::string path = rest.substr(rest.find_first_not_of(" \t") == std::string::npos
                                           ? rest.size()
                                           : rest.find_first_not_of(" \t"));
        std::ifstream f(path);
        if (!f) {
            say("stderr Error: cannot open %s", path.c_str());
            return 1;
        }
        std::stringstream ss;
        ss << f.rdbuf();
        std::lock_guard<std::recursive_mutex> g(S.mu);
        S.deck = ss.str();
        return 0;
    }
    if (verb == "tran") {
        g_lastTran = rest;
        return do_tran(rest);
    }
    if (verb == "run")
        return do_tran("");
    if (verb == "bg_run" || verb == "bg_tran") {
        if (S.running)
            return 1;
        std::string args = verb == "bg_tran" ? rest : "";
        start_bg([args] { do_tran(args); });
        return 0;
    }
    if (verb == "bg_halt" || verb == "halt") {
        /* the background run stops at the end of its current window, with
         * its state kept on the device (sharedspice.c bg_halt) */
        S.haltReq = true;
        if (S.bg.joinable())
            S.bg.join();
        S.haltReq = false;
        return 0;
    }
    if (verb == "bg_resume" || verb == "resume") {
        if (S.running)
            return 1;
        if (!S.active)
            return 0;   /* nothing halted: the run had already ended */
        if (verb == "resume") {
            bool halted = false;
            return continue_tran(&halted);
        }
        start_bg([] {
            bool halted = false;
            continue_tran(&halted);
        });
        return 0;
    }
    if (verb == "remcirc" || verb == "destroy" || verb == "reset") {
        std::lock_guard<std::recursive_mutex> g(S.mu);
        if (verb == "remcirc")
            S.deck.clear();
        if (verb == "destroy")
            S.plots.clear(), S.cur = -1;
        return 0;
    }
    if (verb == "echo") {
        say("stdout %s", rest.c_str());
        return 0;
    }
    if (verb == "quit" || verb == "exit") {
        if (S.ngexit)
            S.ngexit(0, false, true, S.ident, S.user);
        return 0;
    }
    if (verb == "set" || verb == "unset" || verb == "option" || verb == "setplot") {
        if (verb == "setplot") {
            std::string nm;
            std::istringstream r(rest);
            r >> nm;
            for (size_t i = 0; i < S.plots.size(); i++)
                if (S.plots[i]->name == nm)
                    S.cur = (int)i;
        }
        return 0;
    }
    say("stderr Error: unsupported command %s", verb.c_str());
    return 1;
}

}  // namespace

extern "C" {

IMPEXP int ngSpice_Init(SendChar *printfcn, SendStat *statfcn, ControlledExit *ngexit,
                        SendData *sdata, SendInitData *sinitdata, BGThreadRunning *bgtrun,
                        void *userData)
{
    std::lock_guard<std::recursive_mutex> g(S.mu);
    S.pfcn = printfcn;
    S.statfcn = statfcn;
    S.ngexit = ngexit;
    S.datfcn = sdata;
    S.initfcn = sinitdata;
    S.bgfcn = bgtrun;
    S.user = userData;
    return 0;
}

IMPEXP int ngSpice_Init_Sync(GetVSRCData *vsrcdat, GetISRCData *isrcdat, GetSyncData *syncdat,
                             int *ident, void *userData)
{
    (void)vsrcdat;
    (void)isrcdat;
    std::lock_guard<std::recursive_mutex> g(S.mu);
    S.syncfcn = syncdat;
    if (ident)
        S.ident = *ident;
    if (userData)
        S.user = userData;
    return 0;
}

IMPEXP int ngSpice_Command(char *cmd)
{
    if (!cmd) {
        /* NULL command: the reference clears its internal state */
        return 0;
    }
    try {
        return command(cmd);
    } catch (const std::exception &e) {
        say("stderr Error: %s", e.what());
        return 1;
    }
}

IMPEXP pvector_info ngGet_Vec_Info(char *vecname)
{
    if (!vecname)
        return nullptr;
    std::lock_guard<std::recursive_mutex> g(S.mu);
    if (S.cur < 0)
        return nullptr;
    std::string nm = lower(vecname);
    /* accept v(node) and i(source) the way vector lookup does */
    if (nm.size() > 3 && nm[1] == '(' && nm.back() == ')') {
        std::string inner = nm.substr(2, nm.size() - 3);
        if (nm[0] == 'v')
            nm = inner;
        else if (nm[0] == 'i')
            nm = inner + "#branch";
    }
    for (auto &v : S.plots[S.cur]->vecs)
        if (v->name == nm)
            return &v->info;
    return nullptr;
}

IMPEXP int ngSpice_Circ(char **circarray)
{
    if (!circarray)
        return 1;
    std::ostringstream os;
    for (int i = 0; circarray[i]; i++)
        os << circarray[i] << "\n";
    std::lock_guard<std::recursive_mutex> g(S.mu);
    S.deck = os.str();
    return 0;
}

IMPEXP char *ngSpice_CurPlot(void)
{
    std::lock_guard<std::recursive_mutex> g(S.mu);
    static std::string name;
    name = S.cur >= 0 ? S.plots[S.cur]->name : "const";
    return (char *)name.c_str();
}

IMPEXP char **ngSpice_AllPlots(void)
{
    std::lock_guard<std::recursive_mutex> g(S.mu);
    S.nameStore.clear();
    for (auto it = S.plots.rbegin(); it != S.plots.rend(); ++it)
        S.nameStore.push_back((*it)->name);
    S.nameStore.push_back("const");
    S.nameList.clear();
    for (auto &s : S.nameStore)
        S.nameList.push_back((char *)s.c_str());
    S.nameList.push_back(nullptr);
    return S.nameList.data();
}

IMPEXP char **ngSpice_AllVecs(char *plotname)
{
    std::lock_guard<std::recursive_mutex> g(S.mu);
    S.nameStore.clear();
    for (auto &p : S.plots)
        if (plotname && p->name == plotname)
            for (auto &v : p->vecs)
                S.nameStore.push_back(v->name);
    S.nameList.clear();
    for (auto &s : S.nameStore)
        S.nameList.push_back((char *)s.c_str());
    S.nameList.push_back(nullptr);
    return S.nameList.data();
}

IMPEXP NG_BOOL ngSpice_running(void) { return S.running; }

IMPEXP NG_BOOL ngSpice_SetBkpt(double time)
{
    std::lock_guard<std::recursive_mutex> g(S.mu);
    S.extraBreaks.push_back(time);
    return false;   /* breakpoints set from the host are not forwarded to a run */
}

IMPEXP int ngSpice_nospinit(void) { return 0; }
IMPEXP int ngSpice_nospiceinit(void) { return 0; }
IMPEXP int ngSpice_LockRealloc(void)
{
    S.mu.lock();
    return 0;
}
IMPEXP int ngSpice_UnlockRealloc(void)
{
    S.mu.unlock();
    return 0;
}
IMPEXP int ngSpice_Reset(void)
{
    if (S.bg.joinable())
        S.bg.join();
    std::lock_guard<std::recursive_mutex> g(S.mu);
    S.deck.clear();
    S.plots.clear();
    S.cur = -1;
    return 0;
}

}  // extern "C"

/* ------------------------------------------------------------------ */
/* Operator surface: SMPreorder and the device-type table              */
/* ------------------------------------------------------------------ */
extern "C" {

NGSF_API int ngsf_smp_reorder(ngsf_handle *h, double pivtol, double pivrel, double diag_gmin)
{
    if (!h || !h->p.dev)
        return fail("ngsf_smp_reorder: null or host-only handle");
    try {
        Prepared &p = h->p;
        std::vector<double> ax = p.dev->read_ax();
        /* the factorization sees gmin on every structural diagonal
         * (LoadGmin, src/maths/KLU/klusmp.c:762-764) */
        if (diag_gmin != 0.0)
            for (int j = 0; j < p.img.n; j++)
                if (p.img.a_diag[j] >= 0)
                    ax[p.img.a_diag[j]] += diag_gmin;
        if (!plan_lu(p.img.n, p.img.a_cp, p.img.a_ri, ax, pivrel, pivtol, p.img, g_err))
            return NGSF_E_SINGULAR;
        p.dev->upload_lu(p.img);
    } catch (const std::exception &e) {
        return fail(std::string("ngsf_smp_reorder: ") + e.what());
    }
    return ngsf_internal_lufac(h, diag_gmin);
}

NGSF_API int ngsf_smp_preorder(const ngsf_handle *h, int *nblocks, int *largest_block)
{
    if (!h)
        return fail("ngsf_smp_preorder: null handle");
    int nb = 0, big = 0;
    if (!btf_analyze(h->p.img.n, h->p.img.a_cp, h->p.img.a_ri, nb, big))
        return fail("ngsf_smp_preorder: structurally singular matrix");
    if (nblocks)
        *nblocks = nb;
    if (largest_block)
        *largest_block = big;
    return 0;
}

NGSF_API int ngsf_phase_cycles(const ngsf_handle *h, long long *cycles)
{
    const ngsf_ckt_t *d = ngsf_internal_desc(h);
    if (!d || !cycles)
        return fail("ngsf_phase_cycles: null handle or buffer");
    if (!d->prof)
        return fail("ngsf_phase_cycles: the circuit was opened without NGSF_PHASES=1");
    cudaError_t e = cudaMemcpy(cycles, d->prof, NGSF_P_COUNT * sizeof(long long),
                               cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return fail(std::string("ngsf_phase_cycles: ") + cudaGetErrorString(e));
    return 0;
}

static const ngsf_devinfo g_devtable[NGSF_DEV_TYPES] = {
    /* name, states/instance, stamp slots/instance, load, trunc, accept */
    {"BSIM4", B4S_COUNT, B4_NSTAMP, 1, 1, 0},
    {"Capacitor", 2, 6, 1, 1, 0},
    {"Diode", DIS_COUNT, DIO_NSTAMP, 1, 1, 0},
    {"Isource", 0, 2, 1, 0, 1},
    {"Mos1", M1S_COUNT, M1_NSTAMP, 1, 1, 0},
    {"Resistor", 0, 4, 1, 0, 0},
    {"Vsource", 0, 5, 1, 0, 1},
};

NGSF_API int ngsf_dev_table(int *count, const ngsf_devinfo **table)
{
    if (count)
        *count = NGSF_DEV_TYPES;
    if (table)
        *table = g_devtable;
    return 0;
}

}  // extern "C"

