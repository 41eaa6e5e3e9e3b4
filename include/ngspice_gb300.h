/*
 * Engine-level C ABI of the GB300 transient engine: the operator surface
 * underneath the sharedspice API (sharedspice.h), for callers that drive
 * circuits directly and for the parity tests.
 *
 * Reference interfaces each entry point replaces:
 *   ngsf_open     netlist -> circuit: INPpas1/INPpas2 (src/spicelib/parser/
 *                 inppas1.c, inppas2.c), CKTsetup (src/spicelib/analysis/
 *                 cktsetup.c:34), CKTtemp, SMPpreOrder + SMPreorder
 *                 (src/maths/KLU/klusmp.c:1256, :753) on the first stamped
 *                 matrix
 *   ngsf_open_many  ngsf_open for a batch (Monte Carlo instances, corners):
 *                 the parse/setup half on all host cores
 *   ngsf_run      CKTdoJob -> DCtran (src/spicelib/analysis/dctran.c:67) with
 *                 CKTload/DEVload, SMPluFac, SMPsolve, NIconvTest, CKTtrunc on
 *                 the GPU; many circuits in one launch
 *   ngsf_points   the accepted-point stream CKTdump -> OUTpData
 *                 (src/spicelib/analysis/cktdump.c:33)
 *   ngsf_capture  the stamped matrix and right-hand side of each Newton
 *                 iteration (what NIiter hands to SMPluFac, niiter.c:156)
 * All calls return 0 on success and a nonzero code on failure (NGSF_E_*
 * values of the reference's sperror.h where one applies, -1 otherwise);
 * ngsf_last_error() describes the last failure.
 */
#ifndef NGSPICE_GB300_H
#define NGSPICE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define NGSF_API __attribute__((visibility("default")))

typedef struct ngsf_handle ngsf_handle;

/* Parse, compile, upload and pivot one circuit.  probes: space-separated
 * equation names to record at every accepted point (NULL or "" = all).
 * outcap: accepted points to keep.  capmax: Newton iterations whose
 * stamped system is captured (0 = none).  Returns NULL on error. */
NGSF_API ngsf_handle *ngsf_open(const char *netlist, const char *probes, int outcap,
                                int capmax);
/* ngsf_open for count netlists with the same probes, outcap and capmax:
 * parsing and setup run on all host cores, allocation and upload on the
 * calling thread's device.  On success out[0..count-1] receive the handles
 * and 0 is returned; on any failure nothing is returned in out, -1 is
 * returned and ngsf_last_error() names the failing netlist. */
NGSF_API int ngsf_open_many(const char *const *netlists, int count, const char *probes,
                            int outcap, int capmax, ngsf_handle **out);
/* Host-only compile (parse, setup, temperature; no device, no pivoting):
 * ngsf_info / ngsf_eq_name / ngsf_pattern work on the result, ngsf_run
 * refuses it.  Replaces the reference's INPpas1/INPpas2 + CKTsetup +
 * CKTtemp without SMPpreOrder. */
NGSF_API ngsf_handle *ngsf_compile(const char *netlist);
NGSF_API void ngsf_close(ngsf_handle *h);
NGSF_API const char *ngsf_last_error(void);

/* sizes: unknowns, matrix nonzeros, state doubles, L+U nonzeros */
NGSF_API int ngsf_info(const ngsf_handle *h, int *n, int *nnz, int *nstates, int *nlu);
/* name of equation eq (1..n) */
NGSF_API int ngsf_eq_name(const ngsf_handle *h, int eq, char *buf, int len);
/* matrix pattern, CSC: colptr[n+1], rowidx[nnz] (0-based equations - 1) */
NGSF_API int ngsf_pattern(const ngsf_handle *h, int *colptr, int *rowidx);
/* probe list: equation numbers (1..n) of the recorded values */
NGSF_API int ngsf_probes(const ngsf_handle *h, int *eqs, int max);

/* Run .tran on count circuits in one GPU launch.  max_steps bounds the
 * time loop of each circuit.  seconds (may be NULL) receives the device
 * time of the launch. */
NGSF_API int ngsf_run(ngsf_handle *const *hs, int count, long long max_steps,
                      double *seconds);

/* results: ires[14] (status, npoints, accepted, rejected, numIter,
 * tranIter, timePts, ncap, opIter, badPivot, reorders, and with a Newton
 * predictor: steps started from its guess, of those accepted after the
 * first iteration, and retried from the plain start), fres[3] (time
 * reached, last step, diagonal gmin in force) */
NGSF_API int ngsf_results(const ngsf_handle *h, int *ires, double *fres);
/* accepted points: buf[np][1 + nprobe] = time, probe values; returns np */
NGSF_API int ngsf_points(const ngsf_handle *h, double *buf, int maxpoints);
/* captured iterations: ax[k][nnz], rhs[k][n+1], rhsold[k][n+1],
 * meta[k][4] = time, delta, mode, order; returns the count */
NGSF_API int ngsf_capture(ngsf_handle *h, double *ax, double *rhs, double *rhsold,
                          double *meta, int maxcap);
/* floating-point operations of one LU refactorization (multiply-adds) */
NGSF_API double ngsf_lu_flops(const ngsf_handle *h);
/* kernel launches made by the last ngsf_run on this thread (the time loop
 * pauses for host re-pivoting where the reference re-factors) */
NGSF_API int ngsf_last_launches(void);
/* instance counts for roofline accounting: counts[10] = mos1, res, cap,
 * vsrc, isrc, matrix nonzeros, L+U nonzeros, unknowns, bsim4, diode */
NGSF_API int ngsf_workload(const ngsf_handle *h, long long *counts);
/* device bytes held by the circuit */
NGSF_API long long ngsf_device_bytes(const ngsf_handle *h);

/* First-iteration stamps of an opened circuit, with no allocation.
 *
 * No reference counterpart: it evaluates what the reference's first Newton
 * iteration hands to the factorization -- CKTload in MODETRANOP |
 * MODEINITJCT from zero state -- and copies the stamped matrix (ax[nnz], CSC
 * order of ngsf_pattern) and right-hand side (rhs[n+1], rhs[0] = ground) to
 * the caller's host buffers.  The result equals the first matrix and
 * right-hand side ngsf_capture records for the same circuit.
 *
 * Why it exists: the call allocates nothing -- no cudaMalloc/cudaFree and
 * no allocating library routine.  Every array the launch writes lives in one
 * file-scope static device array of the library (8 MiB); the circuit's own
 * device memory is only read.  Callers that cannot allocate device memory
 * when they need the stamps can use it: a process whose device memory is
 * already handed out to a framework's pool, a loop that must not pay for the
 * device-wide synchronisation cudaFree implies, an embedder with a fixed
 * memory budget.
 *
 * Limits and rules:
 * - a circuit whose arrays need more than the 8 MiB is refused: -1, and
 *   ngsf_last_error() names the size it would need;
 * - nothing in the static array has to start at zero: the launch clears the
 *   state vectors, right-hand sides and per-instance memories itself, and
 *   every device rewrites all of its stamp slots;
 * - the first call on a device looks the static array up
 *   (cudaGetSymbolAddress, with that device current) and keeps the address;
 *   make that first call before any stream capture begins;
 * - there is one static array per device: calls that overlap in time (from
 *   several threads, or while an earlier call's work is still running)
 *   race on it and must be serialised by the caller.
 * Returns 0, or -1 with ngsf_last_error() set. */
NGSF_API int ngsf_stamp_initial_static(const ngsf_handle *h, double *ax, double *rhs);

/* ---------------------------------------------------------------------- *
 * Learned Newton predictor: the network kernels (no reference counterpart;
 * the reference's Newton starts from the previous solution and the devices'
 * INITPRED extrapolation, src/maths/ni/niiter.c:29-367).
 *
 * A shared-weight message-passing network over a circuit's node graph (3
 * layers, width 64, BF16 tensor-core products with FP32 accumulation)
 * predicting per node a correction to the linear extrapolation of the node
 * voltage to the next timepoint.  Parameters are an FP32 master copy in a
 * flat layout of ngsf_gnn_param_count() floats: Win[16][64], bin[64],
 * three times (W[128][64], b[64]), Wout[64][16], bout[1].
 * ---------------------------------------------------------------------- */
typedef struct ngsf_gnn ngsf_gnn;

NGSF_API int ngsf_gnn_param_count(void);
/* A network state for one graph of nnodes nodes; neighbour lists in CSR
 * (nbr_ptr[nnodes+1], nbr_idx), symmetric.  NULL on error. */
NGSF_API ngsf_gnn *ngsf_gnn_create(int nnodes, const int *nbr_ptr, const int *nbr_idx);
NGSF_API void ngsf_gnn_destroy(ngsf_gnn *g);
/* set the FP32 master parameters (resets the optimiser); read them back */
NGSF_API int ngsf_gnn_set_params(ngsf_gnn *g, const float *flat);
NGSF_API int ngsf_gnn_get_params(const ngsf_gnn *g, float *flat);
/* X: host [nnodes][16] features; pred: host [nnodes] */
NGSF_API int ngsf_gnn_forward(ngsf_gnn *g, const float *X, float *pred);
/* Forward, loss sum_i w_i (pred_i - y_i)^2 / (2 sum_i w_i), backward and,
 * when lr > 0, one Adam step.  loss and grads (flat layout) are optional
 * host outputs. */
NGSF_API int ngsf_gnn_train_step(ngsf_gnn *g, const float *X, const float *y, const float *w,
                                 float lr, float *loss, float *grads);
/* The tensor-core product on its own: C[M][N] = bf16(A)[M][K] bf16(B)[N][K]^T
 * with FP32 accumulation (host arrays); M % 128 == 0, N % 16 == 0 and
 * N <= 128, K % 16 == 0; the K range split over `splits` blocks. */
NGSF_API int ngsf_gnn_gemm_test(const float *A, const float *B, float *C, int M, int N, int K,
                                int splits);

/* The predictor's view of a circuit: the voltage unknowns (equation
 * indices 1..n, *nv of them), their neighbour lists from the matrix
 * pattern (CSR gptr[nv+1], gidx[*nedges], symmetric), and per node
 * log(1 + count) of incident MOSFET gate, drain/source, bulk, capacitor,
 * resistor and source terminals (stat[nv][6]).  Array arguments may be
 * NULL (sizes first). */
NGSF_API int ngsf_node_graph(const ngsf_handle *h, int *nv, int *nedges, int *vnode, int *gptr,
                             int *gidx, float *stat);
/* Newton predictor for the circuit's next runs: kind 0 off (the
 * reference's start), 1 linear extrapolation of the last two accepted
 * points, 2 that plus the network's correction of the node voltages
 * (params: flat layout above).  With a predictor, Newton at each new
 * timestep starts from its guess, may be accepted after the first
 * iteration when NIconvTest passes, and a start that misses itl4 is
 * retried from the plain start.  Features per node at step n: v_n,
 * (v_n - v_{n-1})/0.05, (v_{n-1} - v_{n-2})/0.05, r1 = h_{n+1}/h_n and
 * r2 = h_n/h_{n-1} (each at most 4), r1 (v_n - v_{n-1})/0.05, stat[6], 1,
 * r1 (r1+1) r2 (d1 - r2 d2) / ((r2+1) 0.05) with d1 = v_n - v_{n-1},
 * d2 = v_{n-1} - v_{n-2}, 0, 0; the guess is v_n + r1 d1 + 0.05 g pred
 * with g = a / (a + 1e-4 V), a = |d1| + |d2| (quiet nodes keep the
 * linear extrapolation). */
NGSF_API int ngsf_set_predictor(ngsf_handle *h, int kind, const float *params);

/* Whether the circuit runs over the whole grid when it is alone or in a
 * batch of at most four (wide), and with how many blocks. */
NGSF_API int ngsf_wide_info(const ngsf_handle *h, int *wide, int *blocks);
/* Shape of the refactorization in a wide launch: the number of blocks that
 * take part (0 = 48) and the work (updates + divisions) at or below which a
 * level runs in one block without a grid barrier (0 = 1024).  Every shape
 * gives the same result; the autotuner (engine.tune_factor_shape) picks
 * the fastest by timing short runs.  No reference counterpart: it is the
 * tuning knob of the GPU refactorization that replaces SMPluFac. */
NGSF_API int ngsf_set_factor_shape(ngsf_handle *h, int blocks, int small_work);

#ifdef __cplusplus
}
#endif
#endif
