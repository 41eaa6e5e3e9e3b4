/* Host runtime of the GPU transient engine; see runtime.cpp. */
#ifndef NGSF_RUNTIME_H
#define NGSF_RUNTIME_H

#include <math.h>
#include <memory>
#include <string>
#include <vector>

#include "circuit.h"
#include "ngsf_types.h"

namespace ngsf {

class DeviceCircuit {
public:
    DeviceCircuit();
    ~DeviceCircuit();
    DeviceCircuit(const DeviceCircuit &) = delete;
    DeviceCircuit &operator=(const DeviceCircuit &) = delete;

    void upload(const Image &img, const std::vector<int> &probes, int outcap, int capmax);
    void upload_lu(const Image &img);
    std::vector<double> read_ax();
    void read_results(std::vector<int> &ires, std::vector<double> &fres);
    void read_points(int npoints, std::vector<double> &out);
    void read_capture(int ncap, std::vector<double> &ax, std::vector<double> &rhs,
                      std::vector<double> &meta);
    void set_pred(const Image &img, int kind, const float *params);
    /* refactorization shape of a wide launch (0 = default) */
    void set_factor_shape(int blocks, int small);
    /* windowed runs: stop at the first accepted point at or after pause_at;
     * resume: continue the saved run instead of starting a fresh one */
    void set_run(double pause_at, bool resume);
    /* synchronised runs: stop at the sharedsync points as well; the
     * caller's answer to a stop goes into the saved control block */
    void set_sync(bool on);
    void sync_reply(double delta, int redo);
    const ngsf_ckt_t &desc() const;
    ngsf_ckt_t *device_desc() const;
    size_t bytes() const;

private:
    struct Impl;
    Impl *impl;
    std::vector<int> probes_;
    int n_ = 0, nnz_ = 0, outcap_ = 0, capmax_ = 0;
};

/* The Newton predictor's view of a circuit: its voltage unknowns (equation
 * indices 1..n), their neighbour lists from the matrix pattern (symmetric,
 * sorted), 1/degree, and per node log(1 + count) of the incident MOSFET
 * gate, drain/source, bulk, capacitor, resistor and source terminals. */
struct PredGraph {
    std::vector<int> vnode, gptr, gidx;
    std::vector<float> dinv, stat;
};
PredGraph pred_graph(const Image &img);

/* A circuit compiled, pivoted and resident on the device. */
struct Prepared {
    std::unique_ptr<Circuit> ckt;
    Image img;
    std::vector<int> probes;
    std::unique_ptr<DeviceCircuit> dev;
    std::vector<int> ires;
    std::vector<double> fres;
    std::vector<double> points;   /* [npoints][1 + nprobe] */
    bool wide = false;            /* run alone over a cooperative grid */
    int wide_blocks = 0;
    bool paused = false;          /* stopped at the end of a window, resumable */
};

void prepare(Prepared &p, const std::string &netlist, const std::vector<std::string> &probes,
             int outcap, int capmax);
/* the two halves of prepare(): parse, compile and resolve the probes (host
 * only, safe to run for different circuits on different threads), then
 * allocate and upload on the calling thread's device */
void prepare_host(Prepared &p, const std::string &netlist, const std::vector<std::string> &probes);
void prepare_device(Prepared &p, int outcap, int capmax);
/* Run the transients of cs.  pause_at: stop each circuit at its first
 * accepted point at or after this time (+inf: run to tstop); continuing:
 * circuits paused by an earlier window resume where they stopped, the
 * others start fresh (otherwise every circuit starts fresh). */
int run_batch(const std::vector<Prepared *> &cs, long long maxSteps, double *seconds,
              int *launches = nullptr, double pause_at = INFINITY, bool continuing = false);

}  // namespace ngsf

#endif
