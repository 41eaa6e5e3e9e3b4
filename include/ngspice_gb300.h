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

/* Windowed run (the reference's `stop when` / `resume`, src/spicelib/
 * analysis/dctran.c:334-353 and :454-458): advance each circuit's
 * transient to its first accepted point at or after t_until, then stop,
 * keeping the whole run state on the device.  A circuit stopped by an
 * earlier window continues where it stopped; any other starts a fresh
 * run.  A stopped circuit reports status -3 (paused) in ngsf_results,
 * with the points so far in ngsf_points; one that reached tstop reports
 * 0.  ngsf_run always starts fresh. */
NGSF_API int ngsf_run_window(ngsf_handle *const *hs, int count, double t_until,
                             long long max_steps, double *seconds);

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
 * - every call looks the static array up on the current device
 *   (cudaGetSymbolAddress), so the address is right after a device reset
 *   too; every call copies its results with blocking cudaMemcpy and ends
 *   with cudaDeviceSynchronize, so make calls outside any stream capture;
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
 * points, 3 the quadratic (the parabola through the last three), 2 the
 * quadratic plus the network's correction of the node voltages (params:
 * flat layout above).  With a predictor, Newton at each new
 * timestep starts from its guess, may be accepted after the first
 * iteration when the first solve's node voltages pass NIconvTest against
 * the guess (the point accepted then keeps the guessed voltages, the
 * linearisation point, with the solved branch currents), and a start that
 * misses itl4 is retried from the plain start.  Features per node at step n: v_n,
 * (v_n - v_{n-1})/0.05, (v_{n-1} - v_{n-2})/0.05, r1 = h_{n+1}/h_n and
 * r2 = h_n/h_{n-1} (each at most 4), r1 (v_n - v_{n-1})/0.05, stat[6], 1,
 * r1 (r1+1) r2 (d1 - r2 d2) / ((r2+1) 0.05) with d1 = v_n - v_{n-1},
 * d2 = v_{n-1} - v_{n-2}, 0, 0; the guess is v_n + r1 d1 + r1 (r1+1) r2
 * (d1 - r2 d2) / (r2+1) + 0.005 g pred with g = a / (a + 1e-4 V),
 * a = |d1| + |d2| (quiet nodes keep the quadratic extrapolation). */
NGSF_API int ngsf_set_predictor(ngsf_handle *h, int kind, const float *params);

/* Synchronised runs: the step hand-over of the reference's shared library
 * (GetSyncData through sharedsync, src/sharedspice.c:2437-2490, called
 * from src/spicelib/analysis/dctran.c:598-601 and :937-960).  With sync on,
 * ngsf_run_window also stops (status -3) at every point where the
 * reference calls sharedsync; ngsf_sync_point reports the stop and
 * ngsf_sync_reply hands back the caller's delta and return value before
 * the next ngsf_run_window continues the run.  A stop costs a kernel exit
 * and relaunch, so synchronised runs suit single circuits driven step by
 * step; a batch keeps sync off. */
NGSF_API int ngsf_set_sync(ngsf_handle *h, int on);
/* 1 when h is stopped at a sync point, else 0.  *loc: 0 before a step
 * (after the breakpoint adjustment of delta), 1 after the step's Newton
 * and truncation-error verdict; *redostep: 1 when the engine rejected the
 * step (its time is then already moved back); *time, *delta: CKTtime and
 * CKTdelta; *olddelta: the step just tried (0 at loc 0).  Any pointer may
 * be NULL. */
NGSF_API int ngsf_sync_point(const ngsf_handle *h, int *loc, int *redostep, double *time,
                             double *delta, double *olddelta);
/* The caller's answer: the delta of the next step (> 0) and 1 to redo the
 * step (at loc 1 an accepted step is then discarded and counted as
 * rejected; at loc 0 the reference only counts a rejection). */
NGSF_API int ngsf_sync_reply(ngsf_handle *h, double delta, int redo);

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

/* ---------------------------------------------------------------------- *
 * Operator surface: the device-plugin and matrix calls of one Newton
 * iteration, one at a time on an opened circuit's device arrays, outside
 * ngsf_run.  They replace
 *   CKTload / DEVload    src/spicelib/analysis/cktload.c:32-180 and the
 *                        SPICEdev DEVload entries (src/include/ngspice/
 *                        devdefs.h:50-129), device types in the table
 *                        order of src/spicelib/devices/dev.c:142-200
 *   CKTtrunc / DEVtrunc  src/spicelib/analysis/ckttrunc.c:20-57
 *   NIconvTest           src/maths/ni/niconv.c:21-90
 *   SMPreorder           src/maths/KLU/klusmp.c:753-806 (smpdefs.h:61-86)
 *   SMPluFac             src/maths/KLU/klusmp.c:574-624
 *   SMPsolve             src/maths/KLU/klusmp.c:951-1011
 * Each call is synchronous (it returns after the device work and the
 * copies) and leaves the circuit's arrays as the operation left them; a
 * later ngsf_run starts its transient from scratch.  Matrices are in the
 * CSC order of ngsf_pattern; right-hand sides and solutions are n+1
 * doubles with entry 0 the ground.  Not for concurrent use on one circuit.
 * ---------------------------------------------------------------------- */

/* device types, in the reference's device-table order; bit k of a `types`
 * mask selects type k */
enum {
    NGSF_DEV_BSIM4, NGSF_DEV_CAP, NGSF_DEV_DIO, NGSF_DEV_ISRC, NGSF_DEV_MOS1,
    NGSF_DEV_RES, NGSF_DEV_VSRC, NGSF_DEV_TYPES
};
#define NGSF_DEV_ALL ((1 << NGSF_DEV_TYPES) - 1)

/* One row of the device table: the SPICEdev entries each type has on the
 * GPU (DEVload always; DEVtrunc for the charge-storing types; DEVaccept
 * for the sources, whose breakpoints the transient kernel sets). */
typedef struct {
    const char *name;       /* DEVpublic.name of the reference */
    int states;             /* state doubles per instance (DEVinfo numStates) */
    int stamps;             /* stamp slots per instance */
    int has_load, has_trunc, has_accept;
} ngsf_devinfo;
NGSF_API int ngsf_dev_table(int *count, const ngsf_devinfo **table);

/* The control scalars of a CKTcircuit that a load, a truncation-error
 * estimate or a factorization reads. */
typedef struct {
    double time;            /* CKTtime */
    double delta;           /* CKTdelta */
    double deltaOld[3];     /* CKTdeltaOld[0..2] */
    double ag[3];           /* CKTag[0..2] (NIcomCof; ag[2]: Gear order 2) */
    double gmin;            /* CKTgmin (junction gmin of the devices) */
    double srcFact;         /* CKTsrcFact (source stepping) */
    double diagGmin;        /* CKTdiagGmin (added to the diagonal when factoring) */
    int mode;               /* CKTmode bits */
    int order;              /* CKTorder */
} ngsf_point;

/* CKTload at a linearisation point: the device loads of the types in
 * `types` (NGSF_DEV_ALL: every device, the whole CKTload) evaluated at
 * rhsOld[n+1] with CKTstates[0..nvec-1] = states[nvec][nstates] and, for
 * BSIM4, the gate voltage of the last iteration's limiting (BSIM4von,
 * von[BSIM4 instances in load order]).  Any of rhsOld, states, von may be
 * NULL to keep the circuit's current values.  Writes the stamped matrix
 * ax[nnz] and right-hand side rhs[n+1]; *noncon (may be NULL) receives
 * the devices' non-convergence flag (CKTnoncon != 0).  The load updates
 * the circuit's state vectors as the reference's does (read them back
 * with ngsf_ckt_read_states). */
NGSF_API int ngsf_ckt_load(ngsf_handle *h, const ngsf_point *pt, int types,
                           const double *rhsOld, const double *states, int nvec,
                           const double *von, double *ax, double *rhs, int *noncon);
/* the circuit's state vectors CKTstates[0..nvec-1] -> states[nvec][nstates] */
NGSF_API int ngsf_ckt_read_states(const ngsf_handle *h, double *states, int nvec);
/* CKTtrunc: the next time step allowed by the local truncation error of
 * every charge (capacitors, diodes, BSIM4 qb/qg/qd, MOS1 Meyer charges),
 * min(2 * pt->delta, CKTterr over all charges), from CKTstates[0..nvec-1]
 * (order + 2 vectors are read; pt->order 1 or 2, trapezoidal). */
NGSF_API int ngsf_ckt_trunc(ngsf_handle *h, const ngsf_point *pt, const double *states,
                            int nvec, double *timestep);
/* NIconvTest of a new solution rhs against the previous one rhsOld
 * (node voltages against vntol, branch currents against abstol, both
 * plus reltol); *noncon = 1 when any unknown has not converged. */
NGSF_API int ngsf_ni_convtest(ngsf_handle *h, const double *rhs, const double *rhsOld,
                              int *noncon);
/* The device matrix values (what the devices' stamp pointers write into
 * KLU's Ax): set them, or read them back after a load. */
NGSF_API int ngsf_smp_set_matrix(ngsf_handle *h, const double *ax);
NGSF_API int ngsf_smp_get_matrix(const ngsf_handle *h, double *ax);
/* SMPpreOrder's symbolic analysis (klu_analyze with btf = TRUE,
 * src/maths/KLU/klusmp.c SMPpreOrder): the block upper triangular form of
 * the pattern from a maximum transversal and the strongly connected
 * components of the matched graph; *nblocks diagonal blocks, the largest
 * *largest_block unknowns.  Works on host-only handles.  The engine's
 * pivot planner does not use the blocks by default: its Markowitz
 * elimination with singleton rows first already reaches KLU's fill;
 * NGSF_ORDER=klu makes it factor in the BTF order, each block in a
 * minimum degree order, with KLU's diagonal-preferring threshold pivots. */
NGSF_API int ngsf_smp_preorder(const ngsf_handle *h, int *nblocks, int *largest_block);
/* SMPreorder: new pivots from the device matrix (threshold pivoting with
 * pivrel and pivtol, diag_gmin added to every structural diagonal), then
 * the device factorization on them.  Returns 0, NGSF_E_SINGULAR (102), or
 * -1 on an error. */
NGSF_API int ngsf_smp_reorder(ngsf_handle *h, double pivtol, double pivrel, double diag_gmin);
/* SMPluFac: refactor the device matrix on the current pivots (diag_gmin
 * added to the diagonal).  Like klu_refactor it fails only on a zero or
 * non-finite pivot: NGSF_E_SINGULAR, after which ngsf_smp_reorder picks
 * new pivots.  -1 when no pivots exist yet. */
NGSF_API int ngsf_smp_lufac(ngsf_handle *h, double diag_gmin);
/* SMPsolve: rhs[n+1] <- the solution of the factored system, in place. */
NGSF_API int ngsf_smp_solve(ngsf_handle *h, double *rhs);

/* Per-phase SM clock cycles of the circuit's last ngsf_run, as its
 * (first) block saw them: cycles[8] = device loads, stamp gather, LU
 * refactorization, triangular solves, convergence test, truncation-error
 * estimate, the whole run, and the Newton iterations counted.  Recorded
 * only for circuits opened while the environment variable NGSF_PHASES=1
 * is set (a profiling aid, no reference counterpart: the reference keeps
 * STATloadTime / STATdecompTime / STATsolveTime in its statistics,
 * src/include/ngspice/optdefs.h:20-53). */
NGSF_API int ngsf_phase_cycles(const ngsf_handle *h, long long *cycles);

/* Measurement aids (no reference counterpart).  ngsf_eval_bench times the
 * device evaluation half of CKTload on its own: every thread of a grid of
 * `blocks` blocks (0 = one per SM) evaluates the circuit's devices of the
 * types in `types` (BSIM4, MOS1, diode) one instance at a time, `reps`
 * times, at the circuit's current linearisation point with the control
 * scalars of pt; *seconds receives the device time (CUDA events).
 * ngsf_fp64_peak measures the device's FP64 fused-multiply-add
 * throughput (flop/s) with independent chains on every SM. */
NGSF_API int ngsf_eval_bench(ngsf_handle *h, const ngsf_point *pt, int types, int reps,
                             int blocks, double *seconds);
NGSF_API int ngsf_fp64_peak(double *flops_per_second);

#ifdef __cplusplus
}
#endif
#endif
