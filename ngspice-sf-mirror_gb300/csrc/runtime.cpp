/*
 * Host runtime: owns the device copy of compiled circuits and drives the
 * GPU transient engine.
 *
 * One run of `.tran` on a circuit goes:
 *   1. upload the compiled image into one device arena;
 *   2. launch: operating point and time loop run on the GPU; the kernel
 *      pauses wherever the reference would re-factor with pivoting
 *      (SMPreorder at MODEINITJCT, the first MODEINITFIX iteration, the
 *      first two iterations after MODEINITTRAN, or a failed refactor);
 *   3. at a pause the host chooses pivots from the stamped matrix
 *      (sparse.cpp), uploads the new LU plan and relaunches; the kernel
 *      resumes from its saved control block;
 *   4. download of accepted points and counters.
 * A batch runs many circuits per launch, one block each; only the paused
 * ones are relaunched.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <system_error>
#include <thread>
#include <atomic>
#include <cstdlib>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "circuit.h"
#include "runtime.h"
#include "bsim4.h"
#include "dio.h"
#include "sparse.h"

extern "C" int ngsf_wide_blocks(void);
extern "C" int ngsf_solve_smem_bytes(int n, int tags);
extern "C" int ngsf_pred_smem_bytes(int any);
extern "C" cudaError_t ngsf_launch_tran_wide(const ngsf_ckt_t *d_ckt, int nblocks, int runMode,
                                             long long maxSteps, int solveCap, int gnnBytes,
                                             cudaStream_t stream);
extern "C" cudaError_t ngsf_launch_tran(const ngsf_ckt_t *d_ckts, const int *d_order, int nckt,
                                        int runMode, long long maxSteps, int solveCap,
                                        int gnnBytes, int threads, cudaStream_t stream);
extern "C" int ngsf_ctl_bytes(void);
extern "C" cudaError_t ngsf_sync_write(void *ctlsave, double delta, int reply);
extern "C" int ngsf_tran_occupancy(int threads, int dynSmem, int *regs, int *smem);

namespace ngsf {

namespace {

void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA error in ") + what + ": " +
                                 cudaGetErrorString(e));
}

/* bump allocator over one device allocation */
struct Arena {
    size_t used = 0;
    std::vector<std::pair<size_t, const void *>> uploads;   /* offset, host src */
    std::vector<size_t> sizes;
    size_t take(size_t bytes)
    {
        size_t off = (used + 255) & ~(size_t)255;
        used = off + bytes;
        return off;
    }
};

}  // namespace

struct DeviceCircuit::Impl {
    char *base = nullptr;
    size_t bytes = 0;
    char *lubase = nullptr;
    size_t lubytes = 0, lucap = 0;
    char *predbase = nullptr;  /* Newton predictor arrays */
    size_t predbytes = 0;
    ngsf_ckt_t h{};            /* device pointers */
    ngsf_ckt_t *d_desc = nullptr;
};

DeviceCircuit::DeviceCircuit() : impl(new Impl) {}
DeviceCircuit::~DeviceCircuit()
{
    if (impl->base)
        cudaFree(impl->base);
    if (impl->lubase)
        cudaFree(impl->lubase);
    if (impl->predbase)
        cudaFree(impl->predbase);
    if (impl->d_desc)
        cudaFree(impl->d_desc);
    delete impl;
}

/* Lay out every array of the image in one arena and copy it up. */
void DeviceCircuit::upload(const Image &img, const std::vector<int> &probes, int outcap,
                           int capmax)
{
    Arena a;
    struct Plan {
        size_t off;
        const void *src;
        size_t bytes;
    };
    std::vector<Plan> plans;
    auto put = [&](const void *src, size_t bytes) -> size_t {
        size_t off = a.take(bytes ? bytes : 8);
        if (src && bytes)
            plans.push_back({off, src, bytes});
        return off;
    };
    auto puti = [&](const std::vector<int> &v) { return put(v.data(), v.size() * sizeof(int)); };
    auto putd = [&](const std::vector<double> &v) {
        return put(v.data(), v.size() * sizeof(double));
    };
    auto zero = [&](size_t bytes) { return put(nullptr, bytes); };

    const int n = img.n;
    const int nnz = (int)img.a_ri.size();
    struct Off {
        size_t b4_node, b4_st, b4_p, b4_h;
        size_t dio_node, dio_st, dio_p;
        size_t mos1_node, mos1_st, mos1_p, mos1_h;
        size_t res_node, res_g;
        size_t cap_node, cap_st, cap_c, cap_m, cap_ic;
        size_t vs[9], is[9];
        size_t ntype, stampv, ax, gptr, gsrc, rptr, rsrc, heavy, hch_ptr, hch_cell, hpart, a_diag, opsave_rhs, opsave_st;
        size_t lux, lvl_ptr, lvl_col, cdiag, cend, cbeg, kptr, kdep, kpos, kseg, upd_dst,
            upd_src, prow, pcol, fl_ptr, fl_row, bl_ptr, bl_row, lr_ptr, lr_col, lr_pos,
            ur_ptr, ur_col, ur_pos, work;
        size_t states, rhs, rhsOld, breaks, out, probe, cap_ax, cap_rhs, cap_meta, result,
            fresult, ctlsave, wide, prof;
    } o{};
    o.b4_node = puti(img.b4_node);
    o.b4_st = puti(img.b4_st);
    o.b4_p = putd(img.b4_p);
    o.b4_h = zero((size_t)B4H_COUNT * img.nb4 * sizeof(double));
    o.dio_node = puti(img.dio_node);
    o.dio_st = puti(img.dio_st);
    o.dio_p = putd(img.dio_p);
    o.mos1_node = puti(img.mos1_node);
    o.mos1_st = puti(img.mos1_st);
    o.mos1_p = putd(img.mos1_p);
    o.mos1_h = zero((size_t)M1H_COUNT * img.nmos1 * sizeof(double));
    o.res_node = puti(img.res_node);
    o.res_g = putd(img.res_g);
    o.cap_node = puti(img.cap_node);
    o.cap_st = puti(img.cap_st);
    o.cap_c = putd(img.cap_c);
    o.cap_m = putd(img.cap_m);
    o.cap_ic = putd(img.cap_ic);
    auto put_src = [&](size_t *s, const std::vector<int> &node, const std::vector<int> &kind,
                       const std::vector<int> &nc, const std::vector<double> &coef,
                       const std::vector<double> &dc, const std::vector<int> &dcg,
                       const std::vector<double> &m, int cnt) {
        s[0] = puti(node);
        s[1] = puti(kind);
        s[2] = puti(nc);
        s[3] = putd(coef);
        s[4] = putd(dc);
        s[5] = puti(dcg);
        s[6] = putd(m);
        s[7] = zero((size_t)cnt * sizeof(double));
    };
    put_src(o.vs, img.vsrc_node, img.vsrc_kind, img.vsrc_ncoef, img.vsrc_coef, img.vsrc_dc,
            img.vsrc_dcgiven, img.vsrc_m, img.nvsrc);
    put_src(o.is, img.isrc_node, img.isrc_kind, img.isrc_ncoef, img.isrc_coef, img.isrc_dc,
            img.isrc_dcgiven, img.isrc_m, img.nisrc);
    o.ntype = puti(img.ntype);
    o.stampv = zero((size_t)img.nstamp * sizeof(double));
    o.ax = zero((size_t)nnz * sizeof(double));
    o.gptr = puti(img.gptr);
    o.gsrc = puti(img.gsrc);
    o.rptr = puti(img.rptr);
    o.rsrc = puti(img.rsrc);
    o.heavy = puti(img.heavy);
    std::vector<int> hch_ptr(1, 0), hch_cell;
    for (size_t h = 0; h < img.heavy.size(); h++) {
        const int p = img.heavy[h];
        const bool isrhs = p < 0;
        const int e = isrhs ? -p - 1 : p;
        const std::vector<int> &ptr = isrhs ? img.rptr : img.gptr;
        const int m = ptr[e + 1] - ptr[e];
        for (int c = 0; c < (m + NGSF_HCHUNK - 1) / NGSF_HCHUNK; c++)
            hch_cell.push_back((int)h);
        hch_ptr.push_back((int)hch_cell.size());
    }
    o.hch_ptr = puti(hch_ptr);
    o.hch_cell = puti(hch_cell);
    o.hpart = zero((size_t)std::max<size_t>(1, hch_cell.size()) * sizeof(double));
    o.a_diag = puti(img.a_diag);
    probes_ = probes;
    o.probe = puti(probes_);   /* the last uploaded array: zero regions follow */
    o.opsave_rhs = zero((size_t)(n + 1) * sizeof(double));
    o.opsave_st = zero((size_t)(img.nstates + 1) * sizeof(double));
    o.work = zero((size_t)(n + 1) * sizeof(double));
    o.states = zero((size_t)4 * (img.nstates + 1) * sizeof(double));
    o.rhs = zero((size_t)(n + 1) * sizeof(double));
    o.rhsOld = zero((size_t)(n + 1) * sizeof(double));
    const int breakcap = 2 + 4 * (img.nvsrc + img.nisrc) + 64;
    o.breaks = zero((size_t)breakcap * sizeof(double));
    o.out = zero((size_t)outcap * (1 + probes.size()) * sizeof(double));
    o.cap_ax = zero((size_t)capmax * nnz * sizeof(double));
    o.cap_rhs = zero((size_t)2 * capmax * (n + 1) * sizeof(double));
    o.cap_meta = zero((size_t)4 * capmax * sizeof(double));
    o.ctlsave = zero((size_t)ngsf_ctl_bytes() + 64);
    o.result = zero(NGSF_R_ALL * sizeof(int));
    o.fresult = zero(NGSF_F_ALL * sizeof(double));
    o.wide = zero(sizeof(ngsf_wide_t));
    o.prof = zero(NGSF_P_COUNT * sizeof(long long));

    if (impl->base)
        cudaFree(impl->base);
    impl->bytes = a.used;
    ck(cudaMalloc(&impl->base, a.used), "cudaMalloc(arena)");
    ck(cudaMemset(impl->base, 0, a.used), "cudaMemset(arena)");
    {
        /* one host image of the arena up to its last uploaded array (zeros
         * between arrays, as the memset left them) and one copy */
        size_t hi = 0;
        for (auto &p : plans)
            hi = std::max(hi, p.off + p.bytes);
        std::vector<char> stage(hi, 0);
        for (auto &p : plans)
            memcpy(stage.data() + p.off, p.src, p.bytes);
        if (hi)
            ck(cudaMemcpy(impl->base, stage.data(), hi, cudaMemcpyHostToDevice),
               "cudaMemcpy(upload)");
    }

    char *b = impl->base;
    auto I = [&](size_t off) { return (int *)(b + off); };
    auto D = [&](size_t off) { return (double *)(b + off); };
    ngsf_ckt_t &h = impl->h;
    memset(&h, 0, sizeof(h));
    h.n = n;
    h.nstates = img.nstates;
    h.nstamp = img.nstamp;
    h.nnz = nnz;
    h.opt = img.opt;
    h.bsim4 = {img.nb4, I(o.b4_node), I(o.b4_st), D(o.b4_p), D(o.b4_h), img.b4_stamp0};
    h.dio = {img.ndio, I(o.dio_node), I(o.dio_st), D(o.dio_p), nullptr, img.dio_stamp0};
    h.mos1 = {img.nmos1, I(o.mos1_node), I(o.mos1_st), D(o.mos1_p), D(o.mos1_h),
              img.mos1_stamp0};
    h.res = {img.nres, I(o.res_node), D(o.res_g), img.res_stamp0};
    h.cap = {img.ncap, I(o.cap_node), I(o.cap_st), D(o.cap_c), D(o.cap_m), D(o.cap_ic),
             img.cap_stamp0};
    h.vsrc = {img.nvsrc, I(o.vs[0]), I(o.vs[1]), I(o.vs[2]), D(o.vs[3]), D(o.vs[4]),
              I(o.vs[5]), D(o.vs[6]), D(o.vs[7]), img.vsrc_stamp0};
    h.isrc = {img.nisrc, I(o.is[0]), I(o.is[1]), I(o.is[2]), D(o.is[3]), D(o.is[4]),
              I(o.is[5]), D(o.is[6]), D(o.is[7]), img.isrc_stamp0};
    h.ntype = I(o.ntype);
    h.stampv = D(o.stampv);
    h.ax = D(o.ax);
    h.gptr = I(o.gptr);
    h.gsrc = I(o.gsrc);
    h.rptr = I(o.rptr);
    h.rsrc = I(o.rsrc);
    h.nheavy = (int)img.heavy.size();
    h.heavy = I(o.heavy);
    h.nhchunk = (int)hch_cell.size();
    h.hch_ptr = I(o.hch_ptr);
    h.hch_cell = I(o.hch_cell);
    h.hpart = D(o.hpart);
    h.a_diag = I(o.a_diag);
    h.opsave_rhs = D(o.opsave_rhs);
    h.opsave_st = D(o.opsave_st);
    h.work = D(o.work);
    h.states = D(o.states);
    h.rhs = D(o.rhs);
    h.rhsOld = D(o.rhsOld);
    h.breaks = D(o.breaks);
    h.breakcap = breakcap;
    h.out = D(o.out);
    h.probe = I(o.probe);
    h.nprobe = (int)probes.size();
    h.outcap = outcap;
    h.cap_lux = D(o.cap_ax);
    h.cap_rhs = D(o.cap_rhs);
    h.cap_meta = D(o.cap_meta);
    h.capmax = capmax;
    h.ctlsave = (void *)(b + o.ctlsave);
    h.result = I(o.result);
    h.fresult = D(o.fresult);
    h.wide = (ngsf_wide_t *)(b + o.wide);
    /* NGSF_PHASES=1: record per-phase clock cycles (ngsf_phase_cycles) */
    const char *ph = getenv("NGSF_PHASES");
    h.prof = (ph && atoi(ph) != 0) ? (long long *)(b + o.prof) : nullptr;
    h.pause_at = INFINITY;
    h.run_resume = 0;
    /* transient re-pivot rules: the retry after a Newton failure takes new
     * pivots (NGSF_RETRY_REPIVOT=0 turns it off); L growth past a limit
     * (NGSF_TRAN_GROWTH, off by default) */
    h.retry_repivot = 1;
    if (const char *r = getenv("NGSF_RETRY_REPIVOT"))
        h.retry_repivot = atoi(r) != 0;
    h.tran_growth = 0.0;
    if (const char *g = getenv("NGSF_TRAN_GROWTH"))
        h.tran_growth = atof(g);
    /* triangular solves level by level; NGSF_SOLVE=sf: dependency driven
     * (the same bits, measured slower: every row waits term by term on
     * the rows it reads, where a level's rows are fetched ahead of the
     * barrier) */
    h.solve_sf = 0;
    if (const char *sv = getenv("NGSF_SOLVE"))
        h.solve_sf = std::string(sv) == "sf";
    if (!impl->d_desc)
        ck(cudaMalloc(&impl->d_desc, sizeof(ngsf_ckt_t)), "cudaMalloc(desc)");
    ck(cudaMemcpy(impl->d_desc, &h, sizeof(h), cudaMemcpyHostToDevice), "cudaMemcpy(desc)");
    n_ = n;
    nnz_ = nnz;
    outcap_ = outcap;
    capmax_ = capmax;
}

void DeviceCircuit::set_run(double pause_at, bool resume)
{
    ngsf_ckt_t &h = impl->h;
    if (h.pause_at == pause_at && h.run_resume == (resume ? 1 : 0))
        return;
    h.pause_at = pause_at;
    h.run_resume = resume ? 1 : 0;
    ck(cudaMemcpy(impl->d_desc, &h, sizeof(h), cudaMemcpyHostToDevice), "cudaMemcpy(desc)");
}

void DeviceCircuit::set_sync(bool on)
{
    impl->h.sync = on ? 1 : 0;
    if (impl->d_desc)
        ck(cudaMemcpy(impl->d_desc, &impl->h, sizeof(impl->h), cudaMemcpyHostToDevice),
           "cudaMemcpy(desc)");
}

void DeviceCircuit::sync_reply(double delta, int redo)
{
    ck(ngsf_sync_write(impl->h.ctlsave, delta, redo), "sync reply");
}

void DeviceCircuit::set_factor_shape(int blocks, int small)
{
    impl->h.rl_blocks = blocks > 0 ? blocks : 0;
    impl->h.rl_small = small > 0 ? small : 0;
    if (impl->d_desc)
        ck(cudaMemcpy(impl->d_desc, &impl->h, sizeof(impl->h), cudaMemcpyHostToDevice),
           "cudaMemcpy(desc)");
}

const ngsf_ckt_t &DeviceCircuit::desc() const { return impl->h; }
ngsf_ckt_t *DeviceCircuit::device_desc() const { return impl->d_desc; }
size_t DeviceCircuit::bytes() const
{
    return impl->bytes + impl->lubytes + impl->predbytes;
}

namespace {
uint16_t to_bf16(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u)
        return (uint16_t)((u >> 16) | 0x40);      /* quiet NaN */
    u += 0x7fffu + ((u >> 16) & 1u);              /* round to nearest even */
    return (uint16_t)(u >> 16);
}
}  // namespace

PredGraph pred_graph(const Image &img)
{
    PredGraph g;
    const int n = img.n;
    std::vector<int> pos(n + 1, -1);
    for (int k = 1; k <= n; k++)
        if (img.names[k - 1].find("#branch") == std::string::npos) {
            pos[k] = (int)g.vnode.size();
            g.vnode.push_back(k);
        }
    const int nv = (int)g.vnode.size();
    std::vector<std::vector<int>> nb(nv);
    for (int j = 0; j < n; j++) {
        const int pj = pos[j + 1];
        if (pj < 0)
            continue;
        for (int q = img.a_cp[j]; q < img.a_cp[j + 1]; q++) {
            const int pi = pos[img.a_ri[q] + 1];
            if (pi >= 0 && pi != pj) {
                nb[pi].push_back(pj);
                nb[pj].push_back(pi);
            }
        }
    }
    g.gptr.assign(nv + 1, 0);
    g.dinv.assign(nv, 0.0f);
    for (int v = 0; v < nv; v++) {
        std::sort(nb[v].begin(), nb[v].end());
        nb[v].erase(std::unique(nb[v].begin(), nb[v].end()), nb[v].end());
        g.gidx.insert(g.gidx.end(), nb[v].begin(), nb[v].end());
        g.gptr[v + 1] = (int)g.gidx.size();
        if (!nb[v].empty())
            g.dinv[v] = 1.0f / (float)nb[v].size();
    }
    std::vector<int> cnt((size_t)nv * 6, 0);
    auto add = [&](int node, int col) {
        if (node > 0 && node <= n && pos[node] >= 0)
            cnt[(size_t)pos[node] * 6 + col]++;
    };
    for (int i = 0; i < img.nb4; i++) {
        add(img.b4_node[B4N_G * img.nb4 + i], 0);
        add(img.b4_node[B4N_D * img.nb4 + i], 1);
        add(img.b4_node[B4N_S * img.nb4 + i], 1);
        add(img.b4_node[B4N_B * img.nb4 + i], 2);
    }
    for (int i = 0; i < img.nmos1; i++) {
        add(img.mos1_node[M1N_G * img.nmos1 + i], 0);
        add(img.mos1_node[M1N_D * img.nmos1 + i], 1);
        add(img.mos1_node[M1N_S * img.nmos1 + i], 1);
        add(img.mos1_node[M1N_B * img.nmos1 + i], 2);
    }
    for (int i = 0; i < img.ndio; i++) {
        add(img.dio_node[DIN_POS * img.ndio + i], 1);
        add(img.dio_node[DIN_NEG * img.ndio + i], 1);
    }
    for (int i = 0; i < img.ncap; i++) {
        add(img.cap_node[i], 3);
        add(img.cap_node[img.ncap + i], 3);
    }
    for (int i = 0; i < img.nres; i++) {
        add(img.res_node[i], 4);
        add(img.res_node[img.nres + i], 4);
    }
    for (int i = 0; i < img.nvsrc; i++) {
        add(img.vsrc_node[i], 5);
        add(img.vsrc_node[img.nvsrc + i], 5);
    }
    for (int i = 0; i < img.nisrc; i++) {
        add(img.isrc_node[i], 5);
        add(img.isrc_node[img.nisrc + i], 5);
    }
    g.stat.resize(cnt.size());
    for (size_t i = 0; i < cnt.size(); i++)
        g.stat[i] = (float)std::log1p((double)cnt[i]);
    return g;
}

/* Newton predictor: kind 0 off, 1 linear extrapolation, 2 with the network
 * (params: the flat FP32 layout of ngsf_gnn_param_count() floats). */
void DeviceCircuit::set_pred(const Image &img, int kind, const float *params)
{
    if (impl->predbase) {
        cudaFree(impl->predbase);
        impl->predbase = nullptr;
        impl->predbytes = 0;
    }
    ngsf_pred_t &P = impl->h.pred;
    memset(&P, 0, sizeof(P));
    if (kind) {
        PredGraph g = pred_graph(img);
        const int nv = (int)g.vnode.size(), nvpad = (nv + 127) / 128 * 128, n1 = img.n + 1;
        Arena a;
        struct Plan {
            size_t off;
            const void *src;
            size_t bytes;
        };
        std::vector<Plan> plans;
        auto put = [&](const void *src, size_t bytes) {
            size_t o = a.take(std::max<size_t>(bytes, 16));
            if (bytes)
                plans.push_back({o, src, bytes});
            return o;
        };
        /* the network, BF16 transposed copies and FP32 biases */
        std::vector<uint16_t> winT(64 * 16), wT[3], woutT(16 * 64);
        std::vector<float> bias(64 * 4 + 1, 0.0f);
        if (kind == 2) {
            const float *Win = params, *bin = Win + 16 * 64;
            for (int o = 0; o < 64; o++)
                for (int i = 0; i < 16; i++)
                    winT[o * 16 + i] = to_bf16(Win[i * 64 + o]);
            memcpy(&bias[0], bin, 64 * 4);
            const float *L = bin + 64;
            for (int l = 0; l < 3; l++) {
                const float *W = L + l * (128 * 64 + 64);
                wT[l].resize(64 * 128);
                for (int o = 0; o < 64; o++)
                    for (int i = 0; i < 128; i++)
                        wT[l][o * 128 + i] = to_bf16(W[i * 64 + o]);
                memcpy(&bias[64 * (l + 1)], W + 128 * 64, 64 * 4);
            }
            const float *Wout = L + 3 * (128 * 64 + 64);
            for (int o = 0; o < 16; o++)
                for (int i = 0; i < 64; i++)
                    woutT[o * 64 + i] = to_bf16(Wout[i * 16 + o]);
            bias[256] = Wout[64 * 16];
        }
        size_t o_vnode = put(g.vnode.data(), nv * 4), o_gptr = put(g.gptr.data(), (nv + 1) * 4),
               o_gidx = put(g.gidx.data(), g.gidx.size() * 4),
               o_dinv = put(g.dinv.data(), nv * 4), o_stat = put(g.stat.data(), g.stat.size() * 4);
        size_t o_ha = a.take((size_t)nvpad * 64 * 4), o_hb = a.take((size_t)nvpad * 64 * 4);
        size_t o_cur = a.take(n1 * 8), o_h0 = a.take(n1 * 8), o_h1 = a.take(n1 * 8);
        size_t o_win = put(winT.data(), kind == 2 ? winT.size() * 2 : 0), o_w[3];
        for (int l = 0; l < 3; l++)
            o_w[l] = put(wT[l].data(), wT[l].size() * 2);
        size_t o_wout = put(woutT.data(), kind == 2 ? woutT.size() * 2 : 0);
        size_t o_bias = put(bias.data(), bias.size() * 4);
        ck(cudaMalloc(&impl->predbase, a.used), "cudaMalloc(predictor)");
        ck(cudaMemset(impl->predbase, 0, a.used), "cudaMemset(predictor)");
        impl->predbytes = a.used;
        for (auto &pl : plans)
            ck(cudaMemcpy(impl->predbase + pl.off, pl.src, pl.bytes, cudaMemcpyHostToDevice),
               "cudaMemcpy(predictor)");
        char *b = impl->predbase;
        P.kind = kind;
        P.nv = nv;
        P.vnode = (const int *)(b + o_vnode);
        P.gptr = (const int *)(b + o_gptr);
        P.gidx = (const int *)(b + o_gidx);
        P.dinv = (const float *)(b + o_dinv);
        P.stat = (const float *)(b + o_stat);
        P.Ha = (float *)(b + o_ha);
        P.Hb = (float *)(b + o_hb);
        P.cur = (double *)(b + o_cur);
        P.h0 = (double *)(b + o_h0);
        P.h1 = (double *)(b + o_h1);
        P.WinT = (const unsigned short *)(b + o_win);
        for (int l = 0; l < 3; l++)
            P.WT[l] = (const unsigned short *)(b + o_w[l]);
        P.WoutT = (const unsigned short *)(b + o_wout);
        const float *bb = (const float *)(b + o_bias);
        P.bin = bb;
        for (int l = 0; l < 3; l++)
            P.bl[l] = bb + 64 * (l + 1);
        P.bout = bb + 256;
    }
    ck(cudaMemcpy(impl->d_desc, &impl->h, sizeof(impl->h), cudaMemcpyHostToDevice),
       "cudaMemcpy(desc)");
}

/* Upload the LU plan (pivot sequence, layout, update lists, levels) into
 * its own allocation, replacing the previous plan. */
void DeviceCircuit::upload_lu(const Image &img)
{
    Arena a;
    struct Plan {
        size_t off;
        const void *src;
        size_t bytes;
    };
    std::vector<Plan> plans;
    auto put = [&](const void *src, size_t bytes) -> size_t {
        size_t off = a.take(bytes ? bytes : 8);
        if (src && bytes)
            plans.push_back({off, src, bytes});
        return off;
    };
    auto puti = [&](const std::vector<int> &v) { return put(v.data(), v.size() * sizeof(int)); };
    /* the right-looking schedule (two barriers per level, every
     * destination of a level in parallel) is faster than the left-looking
     * one (a column's dependency chain per warp) at every size measured;
     * NGSF_LU=ll selects the left-looking one.  Only the selected
     * schedule's arrays are uploaded. */
    bool rl = img.n > 0;
    if (const char *e = getenv("NGSF_LU"))
        rl = std::string(e) != "ll";
    const std::vector<int> none;
    const bool ll = !rl;
    size_t o_lux = put(nullptr, (size_t)img.nlu * sizeof(double));
    size_t o_a_lupos = puti(img.a_lupos), o_lvl_ptr = puti(ll ? img.lvl_ptr : none),
           o_lvl_col = puti(ll ? img.lvl_col : none), o_cdiag = puti(img.cdiag),
           o_cend = puti(img.cend), o_cbeg = puti(img.cbeg), o_kptr = puti(ll ? img.kptr : none),
           o_kdep = puti(ll ? img.kdep : none), o_kpos = puti(ll ? img.kpos : none),
           o_kseg = puti(ll ? img.kseg : none), o_upd_dst = puti(ll ? img.upd_dst : none),
           o_upd_src = puti(ll ? img.upd_src : none), o_prow = puti(img.prow), o_pcol = puti(img.pcol),
           o_fl_ptr = puti(img.fl_ptr), o_fl_row = puti(img.fl_row), o_bl_ptr = puti(img.bl_ptr),
           o_bl_row = puti(img.bl_row), o_lr_ptr = puti(img.lr_ptr), o_lr_col = puti(img.lr_col),
           o_lr_pos = puti(img.lr_pos), o_ur_ptr = puti(img.ur_ptr), o_ur_col = puti(img.ur_col),
           o_ur_pos = puti(img.ur_pos), o_fh_ptr = puti(img.fh_ptr),
           o_fh_row = puti(img.fh_row), o_bh_ptr = puti(img.bh_ptr), o_bh_row = puti(img.bh_row);
    auto descs = [&](const std::vector<int> &rows, const std::vector<int> &ptr) {
        std::vector<int> d(rows.size() * 4, 0);
        for (size_t r = 0; r < rows.size(); r++) {
            d[4 * r] = rows[r];
            d[4 * r + 1] = ptr[rows[r]];
            d[4 * r + 2] = ptr[rows[r] + 1];
        }
        return d;
    };
    const std::vector<int> fdesc = descs(img.fl_row, img.lr_ptr), bdesc = descs(img.bl_row, img.ur_ptr);
    size_t o_fdesc = puti(fdesc), o_bdesc = puti(bdesc);
    size_t o_lval = put(nullptr, std::max<size_t>(1, img.lr_col.size()) * sizeof(double));
    size_t o_uval = put(nullptr, std::max<size_t>(1, img.ur_col.size()) * sizeof(double));
    /* the packed descriptors below replace ud_dst, ud_p, sc_pos, sc_piv on
     * the device */
    size_t o_rl_ptr = puti(rl ? img.rl_ptr : none), o_rl_col = puti(rl ? img.rl_col : none),
           o_sc_ptr = puti(rl ? img.sc_ptr : none), o_sc_pos = puti(none),
           o_sc_piv = puti(none), o_ud_ptr = puti(rl ? img.ud_ptr : none),
           o_ud_dst = puti(none), o_ud_cptr = puti(rl ? img.ud_cptr : none),
           o_ud_l = puti(rl ? img.ud_l : none), o_ud_u = puti(rl ? img.ud_u : none),
           o_ud_p = puti(none);
    /* packed form of the right-looking schedule */
    std::vector<int> ud_pk, sc_pk;
    if (rl) {
        /* column of each diagonal position, and each position's last
         * destination entry (the schedule lists levels in order) */
        std::vector<int> diagcol(std::max(1, img.nlu), -1), last(std::max(1, img.nlu), -1);
        for (size_t k = 0; k < img.cdiag.size(); k++)
            diagcol[img.cdiag[k]] = (int)k;
        for (size_t d = 0; d < img.ud_dst.size(); d++)
            last[img.ud_dst[d]] = (int)d;
        ud_pk.resize(4 * img.ud_dst.size());
        for (size_t d = 0; d < img.ud_dst.size(); d++) {
            const int c0 = img.ud_cptr[d], dst = img.ud_dst[d];
            const bool more = img.ud_cptr[d + 1] - c0 > 1;
            ud_pk[4 * d] = more ? -(dst + 1) : dst;
            ud_pk[4 * d + 1] = img.ud_l[c0];
            ud_pk[4 * d + 2] = img.ud_u[c0];
            ud_pk[4 * d + 3] = (diagcol[dst] >= 0 && last[dst] == (int)d) ? diagcol[dst] : -1;
        }
        sc_pk.resize(2 * img.sc_pos.size());
        for (size_t e = 0; e < img.sc_pos.size(); e++) {
            sc_pk[2 * e] = img.sc_pos[e];
            sc_pk[2 * e + 1] = img.sc_piv[e];
        }
    }
    size_t o_ud_pk = puti(ud_pk), o_sc_pk = puti(sc_pk);
    size_t o_uinv = put(nullptr, (size_t)std::max(1, img.n) * sizeof(double));
    /* one host image of the arena and one copy; the device arena is kept
     * when the new plan fits it (a re-pivot usually changes the fill a
     * little), so a re-plan costs no cudaFree (which synchronises) */
    std::vector<char> stage(a.used, 0);
    for (auto &p : plans)
        memcpy(stage.data() + p.off, p.src, p.bytes);
    if (!impl->lubase || impl->lucap < a.used) {
        if (impl->lubase)
            cudaFree(impl->lubase);
        impl->lubase = nullptr;
        impl->lucap = a.used + a.used / 4;
        ck(cudaMalloc(&impl->lubase, impl->lucap), "cudaMalloc(lu arena)");
    }
    impl->lubytes = a.used;
    ck(cudaMemcpy(impl->lubase, stage.data(), a.used, cudaMemcpyHostToDevice),
       "cudaMemcpy(lu upload)");
    char *b = impl->lubase;
    auto I = [&](size_t off) { return (int *)(b + off); };
    ngsf_ckt_t &h = impl->h;
    h.nlu = img.nlu;
    h.nlevels = (int)img.lvl_ptr.size() - 1;
    h.nflevels = (int)img.fl_ptr.size() - 1;
    h.nblevels = (int)img.bl_ptr.size() - 1;
    h.lux = (double *)(b + o_lux);
    h.a_lupos = I(o_a_lupos);
    h.lvl_ptr = I(o_lvl_ptr);
    h.lvl_col = I(o_lvl_col);
    h.cdiag = I(o_cdiag);
    h.cend = I(o_cend);
    h.cbeg = I(o_cbeg);
    h.kptr = I(o_kptr);
    h.kdep = I(o_kdep);
    h.kpos = I(o_kpos);
    h.kseg = I(o_kseg);
    h.upd_dst = I(o_upd_dst);
    h.upd_src = I(o_upd_src);
    h.prow = I(o_prow);
    h.pcol = I(o_pcol);
    h.fl_ptr = I(o_fl_ptr);
    h.fl_row = I(o_fl_row);
    h.bl_ptr = I(o_bl_ptr);
    h.bl_row = I(o_bl_row);
    h.lr_ptr = I(o_lr_ptr);
    h.lr_col = I(o_lr_col);
    h.lr_pos = I(o_lr_pos);
    h.ur_ptr = I(o_ur_ptr);
    h.ur_col = I(o_ur_col);
    h.ur_pos = I(o_ur_pos);
    h.fdesc = I(o_fdesc);
    h.bdesc = I(o_bdesc);
    h.lval = (double *)(b + o_lval);
    h.uval = (double *)(b + o_uval);
    h.nlterm = (int)img.lr_col.size();
    h.nuterm = (int)img.ur_col.size();
    h.fh_ptr = I(o_fh_ptr);
    h.fh_row = I(o_fh_row);
    h.bh_ptr = I(o_bh_ptr);
    h.bh_row = I(o_bh_row);
    h.rl_levels = rl ? (int)img.rl_ptr.size() - 1 : 0;
    h.rl_ptr = I(o_rl_ptr);
    h.rl_col = I(o_rl_col);
    h.sc_ptr = I(o_sc_ptr);
    h.sc_pos = I(o_sc_pos);
    h.sc_piv = I(o_sc_piv);
    h.ud_ptr = I(o_ud_ptr);
    h.ud_dst = I(o_ud_dst);
    h.ud_cptr = I(o_ud_cptr);
    h.ud_l = I(o_ud_l);
    h.ud_u = I(o_ud_u);
    h.ud_p = I(o_ud_p);
    h.ud_pk = I(o_ud_pk);
    h.sc_pk = I(o_sc_pk);
    h.uinv = (double *)(b + o_uinv);
    ck(cudaMemcpy(impl->d_desc, &h, sizeof(h), cudaMemcpyHostToDevice), "cudaMemcpy(desc)");
}

std::vector<double> DeviceCircuit::read_ax()
{
    std::vector<double> ax(nnz_);
    ck(cudaMemcpy(ax.data(), impl->h.ax, nnz_ * sizeof(double), cudaMemcpyDeviceToHost),
       "cudaMemcpy(ax)");
    return ax;
}

void DeviceCircuit::read_results(std::vector<int> &ires, std::vector<double> &fres)
{
    ires.resize(NGSF_R_ALL);
    fres.resize(NGSF_F_ALL);
    ck(cudaMemcpy(ires.data(), impl->h.result, NGSF_R_ALL * sizeof(int),
                  cudaMemcpyDeviceToHost), "cudaMemcpy(result)");
    ck(cudaMemcpy(fres.data(), impl->h.fresult, NGSF_F_ALL * sizeof(double),
                  cudaMemcpyDeviceToHost), "cudaMemcpy(fresult)");
}

void DeviceCircuit::read_points(int npoints, std::vector<double> &out)
{
    int np = std::min(npoints, outcap_);
    out.resize((size_t)np * (1 + probes_.size()));
    if (np)
        ck(cudaMemcpy(out.data(), impl->h.out, out.size() * sizeof(double),
                      cudaMemcpyDeviceToHost), "cudaMemcpy(out)");
}

void DeviceCircuit::read_capture(int ncap, std::vector<double> &ax, std::vector<double> &rhs,
                                 std::vector<double> &meta)
{
    int nc = std::min(ncap, capmax_);
    ax.resize((size_t)nc * nnz_);
    rhs.resize((size_t)2 * capmax_ * (n_ + 1));
    meta.resize((size_t)4 * nc);
    if (!nc)
        return;
    ck(cudaMemcpy(ax.data(), impl->h.cap_lux, ax.size() * sizeof(double),
                  cudaMemcpyDeviceToHost), "cudaMemcpy(cap ax)");
    ck(cudaMemcpy(rhs.data(), impl->h.cap_rhs, rhs.size() * sizeof(double),
                  cudaMemcpyDeviceToHost), "cudaMemcpy(cap rhs)");
    ck(cudaMemcpy(meta.data(), impl->h.cap_meta, meta.size() * sizeof(double),
                  cudaMemcpyDeviceToHost), "cudaMemcpy(cap meta)");
}

/* ------------------------------------------------------------------ */
/* Prepared circuit: compile + pivot plan, device resident              */
/* ------------------------------------------------------------------ */
void prepare(Prepared &p, const std::string &netlist, const std::vector<std::string> &probeNames,
             int outcap, int capmax)
{
    prepare_host(p, netlist, probeNames);
    prepare_device(p, outcap, capmax);
}

void prepare_host(Prepared &p, const std::string &netlist, const std::vector<std::string> &probeNames)
{
    p.ckt = parse_netlist(netlist);
    compile(*p.ckt, p.img);
    std::vector<int> probes;
    if (probeNames.empty()) {
        for (int i = 1; i <= p.img.n; i++)
            probes.push_back(i);
    } else {
        for (auto &nm : probeNames) {
            int id = -1;
            for (int i = 0; i < p.img.n; i++)
                if (p.img.names[i] == nm)
                    id = i + 1;
            if (id < 0)
                throw NetlistError("unknown probe " + nm);
            probes.push_back(id);
        }
    }
    p.probes = probes;
}

void prepare_device(Prepared &p, int outcap, int capmax)
{
    p.dev = std::make_unique<DeviceCircuit>();
    p.dev->upload(p.img, p.probes, outcap, capmax);
    /* large circuits may take the whole device (a wide launch) when they
     * run in a small batch; NGSF_WIDE=0/1 overrides the size rule */
    int transistors = p.img.nb4 + p.img.nmos1;
    bool wide = transistors >= 1024;
    if (const char *e = getenv("NGSF_WIDE"))
        wide = atoi(e) != 0;
    p.wide = false;
    p.wide_blocks = 0;
    if (wide) {
        int nb = ngsf_wide_blocks();
        if (nb >= 2) {
            p.wide = true;
            p.wide_blocks = nb;
        }
    }
    p.dev->upload_lu(p.img);     /* empty plan: the first iteration asks for one */
}

/* Run .tran on all circuits: launch; circuits that paused for a re-pivot
 * get new pivots from the matrix they stamped and resume in the next
 * launch, until every circuit has finished. */
int run_batch(const std::vector<Prepared *> &cs, long long maxSteps, double *seconds,
              int *launches, double pause_at, bool continuing)
{
    std::vector<Prepared *> pending(cs.begin(), cs.end());
    bool anyFresh = false;
    for (auto *c : pending) {
        const bool resume = continuing && c->paused;
        anyFresh |= !resume;
        c->dev->set_run(pause_at, resume);
        c->paused = false;
    }
    int mode = 0;   /* RUN_FRESH */
    /* a batch of many circuits fills the device with one block per
     * circuit; only a batch of a few runs its large circuits wide */
    bool allowWide = cs.size() <= 4;
    if (const char *e = getenv("NGSF_WIDE"))
        allowWide = atoi(e) != 0;
    double total = 0;
    int nl = 0;
    ngsf_ckt_t *d = nullptr;
    ck(cudaMalloc(&d, std::max<size_t>(1, cs.size()) * sizeof(ngsf_ckt_t)), "cudaMalloc(descs)");
    int *d_order = nullptr;
    ck(cudaMalloc(&d_order, std::max<size_t>(1, cs.size()) * sizeof(int)), "cudaMalloc(order)");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    /* NGSF_TRACE=1: one line per launch and per re-plan round on stderr */
    const bool trace = getenv("NGSF_TRACE") && atoi(getenv("NGSF_TRACE")) != 0;
    /* NGSF_HOLD=1: batched circuits stop after their first accepted
     * transient step while any circuit of the batch still pauses for new
     * pivots, so the early re-pivots (operating point, MODEINITTRAN) of
     * the whole batch cost short launches; the batch then runs its time
     * loops together.  Off by default. */
    const bool holdPolicy = getenv("NGSF_HOLD") && atoi(getenv("NGSF_HOLD")) != 0;
    /* holding only matters while some circuit is still in its first step */
    bool holdNow = holdPolicy && anyFresh;
    try {
        while (!pending.empty()) {
            if (nl > 256 + 8 * (int)cs.size())
                throw std::runtime_error("too many re-pivot rounds");
            std::vector<ngsf_ckt_t> descs;
            std::vector<Prepared *> wide;
            int maxn = 0, learned = 0, tags = 0;
            for (auto *c : pending) {
                if (c->wide && allowWide) {
                    wide.push_back(c);
                } else {
                    descs.push_back(c->dev->desc());
                    maxn = std::max(maxn, c->img.n);
                    learned |= c->dev->desc().pred.kind == 2;
                    tags |= c->dev->desc().solve_sf;
                }
            }
            if (!descs.empty()) {
                ck(cudaMemcpy(d, descs.data(), descs.size() * sizeof(ngsf_ckt_t),
                              cudaMemcpyHostToDevice), "cudaMemcpy(descs)");
                /* largest circuits first: the block scheduler then starts
                 * them first (longest-processing-time order) */
                std::vector<int> order(descs.size());
                for (size_t i = 0; i < order.size(); i++)
                    order[i] = (int)i;
                std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                    const ngsf_ckt_t &x = descs[a], &y = descs[b];
                    return (long long)x.nnz + 30LL * x.bsim4.n + 8LL * x.mos1.n >
                           (long long)y.nnz + 30LL * y.bsim4.n + 8LL * y.mos1.n;
                });
                ck(cudaMemcpy(d_order, order.data(), order.size() * sizeof(int),
                              cudaMemcpyHostToDevice), "cudaMemcpy(order)");
                const int solveCap = ngsf_solve_smem_bytes(maxn, tags);
                const int gnnBytes = ngsf_pred_smem_bytes(learned);
                /* one 256-thread block per circuit (measured faster than
                 * two 128-thread or four 64-thread circuits sharing an SM:
                 * the refactorization and solves need the threads more than
                 * the FP64-bound device evaluation needs a second circuit
                 * to overlap with).  NGSF_BATCH_THREADS (64, 128, 256)
                 * overrides; the result is the same */
                int threads = 256;
                if (const char *bt = getenv("NGSF_BATCH_THREADS"))
                    threads = atoi(bt);
                cudaEventRecord(e0, 0);
                ck(ngsf_launch_tran(d, d_order, (int)descs.size(), mode | (holdNow ? 4 : 0),
                                   maxSteps, solveCap, gnnBytes, threads, 0), "launch(tran)");
                cudaEventRecord(e1, 0);
                ck(cudaEventSynchronize(e1), "tran");
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                total += ms * 1e-3;
                nl++;
                if (trace) {
                    int regs = 0, smem = 0;
                    const int per = ngsf_tran_occupancy(threads, solveCap + gnnBytes, &regs, &smem);
                    fprintf(stderr, "ngsf: launch %d: %zu circuits, largest n %d, %d threads"
                            " (%d blocks per SM; %d registers, %d + %d shared bytes),%s %.3f ms\n",
                            nl, descs.size(), maxn, threads, per, regs, smem,
                            solveCap + gnnBytes, holdNow ? " hold," : "", ms);
                }
            }
            for (auto *c : wide) {
                /* a fresh hand-over block per launch: command numbers start at 0 */
                ck(cudaMemset(c->dev->desc().wide, 0, sizeof(ngsf_wide_t)), "cudaMemset(wide)");
                int nb = c->wide_blocks;
                cudaEventRecord(e0, 0);
                ck(ngsf_launch_tran_wide(c->dev->device_desc(), nb, mode, maxSteps,
                                        ngsf_solve_smem_bytes(c->img.n, c->dev->desc().solve_sf),
                                        ngsf_pred_smem_bytes(c->dev->desc().pred.kind == 2), 0),
                   "launch(tran wide)");
                cudaEventRecord(e1, 0);
                ck(cudaEventSynchronize(e1), "tran wide");
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                total += ms * 1e-3;
                nl++;
                if (trace)
                    fprintf(stderr, "ngsf: launch %d: wide, n %d, %d blocks, %.3f ms\n", nl,
                            c->img.n, nb, ms);
                int err = 0;
                ck(cudaMemcpy(&err, &c->dev->desc().wide->err, sizeof(int),
                              cudaMemcpyDeviceToHost), "cudaMemcpy(wide err)");
                if (err)
                    throw std::runtime_error("wide launch: a block hand-over wait ran out");
            }
            std::vector<Prepared *> next, replan;
            std::vector<std::vector<double>> axs;
            for (auto *c : pending) {
                c->dev->read_results(c->ires, c->fres);
                if (c->ires[NGSF_R_STATUS] == NGSF_NEED_REORDER) {
                    std::vector<double> ax = c->dev->read_ax();
                    /* the factorization sees gmin on the diagonal (LoadGmin) */
                    double dg = c->fres[NGSF_F_DIAGGMIN];
                    if (dg != 0.0)
                        for (int j = 0; j < c->img.n; j++)
                            if (c->img.a_diag[j] >= 0)
                                ax[c->img.a_diag[j]] += dg;
                    replan.push_back(c);
                    axs.push_back(std::move(ax));
                } else if (c->ires[NGSF_R_STATUS] == NGSF_HELD && c->ires[NGSF_R_SYNCLOC] == 0 &&
                           !(c->fres[NGSF_F_TIME] >= pause_at)) {
                    next.push_back(c);   /* held after its first step */
                } else {
                    /* finished, failed, or stopped at the end of the window
                     * or at a sync point */
                    c->paused = c->ires[NGSF_R_STATUS] == NGSF_HELD;
                    c->dev->read_points(c->ires[NGSF_R_NPOINTS], c->points);
                }
            }
            /* new pivots for every paused circuit, on all host cores (each
             * plan only reads its own matrix and writes its own image) */
            std::vector<int> ok(replan.size(), 0);
            const auto tp = std::chrono::steady_clock::now();
            {
                std::atomic<size_t> cursor{0};
                /* 1 planned, 0 singular, -1 the planner itself failed */
                /* each worker plans a circuit and uploads its plan (a
                 * thread of its own: the calling thread's device made
                 * current first) */
                int dev = 0;
                cudaGetDevice(&dev);
                auto work = [&]() {
                    cudaSetDevice(dev);
                    for (size_t i; (i = cursor.fetch_add(1)) < replan.size();) {
                        Prepared *c = replan[i];
                        std::string err;
                        try {
                            ok[i] = plan_lu(c->img.n, c->img.a_cp, c->img.a_ri, axs[i],
                                            c->img.opt.pivrel, c->img.opt.pivtol, c->img, err);
                            if (ok[i] == 1)
                                c->dev->upload_lu(c->img);
                        } catch (const std::exception &) {
                            ok[i] = -1;
                        }
                    }
                };
                unsigned nt = std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()),
                                                 (unsigned)std::max<size_t>(1, replan.size()));
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
            }
            if (trace && !replan.empty())
                fprintf(stderr, "ngsf: re-plan of %zu circuits: %.3f s host\n", replan.size(),
                        std::chrono::duration<double>(std::chrono::steady_clock::now() - tp).count());
            for (size_t i = 0; i < replan.size(); i++)
                if (ok[i] < 0)
                    throw std::runtime_error("pivot planning or plan upload failed");
            for (size_t i = 0; i < replan.size(); i++) {
                Prepared *c = replan[i];
                if (!ok[i]) {
                    c->ires[NGSF_R_STATUS] = NGSF_E_SINGULAR;
                    continue;
                }
                next.push_back(c);
            }
            pending.swap(next);
            mode = 1;   /* RUN_RESUME */
            holdNow = holdPolicy && !replan.empty();
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(d);
        cudaFree(d_order);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    cudaFree(d_order);
    if (seconds)
        *seconds = total;
    if (launches)
        *launches = nl;
    return 0;
}

}  // namespace ngsf
