/*
 * pelelm_gb300 — GB300-native (sm_103a) replacement of the PelePhysics chemistry reactor that
 * PeleLM drives from PeleLM::advance_chemistry (Source/PeleLM.cpp:5626-5845).
 *
 * Plain C ABI: plain pointers and sizes, no C++ or framework types. All device pointers are
 * CUDA device (or managed) memory owned by the caller; the library only reads and writes
 * them in place. Units inside the reactor are CGS, exactly as the reference passes them
 * (rhoY g/cm^3, rhoH erg/cm^3, T K, forcing per second) — Source/PeleLM.cpp:5736-5746.
 *
 * Every entry point returns 0 (or a non-negative count) on success and a negative value on a
 * usage / CUDA error; pgb_last_error() then describes it. Nothing throws across the ABI and no
 * device code traps.
 */
#ifndef PELELM_GB300_H
#define PELELM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGB_ABI_VERSION 1

typedef struct pgb_reactor pgb_reactor;

/* Mirror of amrex::Array4<T>: element (i,j,k,n) is
 * p[(i-begin[0]) + (j-begin[1])*jstride + (k-begin[2])*kstride + n*nstride]. */
typedef struct {
  void* p;
  long long jstride, kstride, nstride;
  int begin[3];
  int end[3]; /* exclusive, as amrex::Array4::end */
  int ncomp;
} pgb_array4;

/* Mirror of amrex::Box (cell-centred, inclusive smallEnd/bigEnd). */
typedef struct {
  int lo[3];
  int hi[3];
} pgb_box;

/* The arguments of ReactorBase::react for one box (Source/PeleLM.cpp:5752-5757):
 * rY (NUM_SPECIES comps), rY_src (NUM_SPECIES), T, rEner (rho h), rEner_src, FC, mask.
 * mask.p may be NULL (all cells react); mask < 0 marks covered cells, which are skipped
 * (their FC is set to 0), the Source/PeleLM_K.H:66-72 convention. */
typedef struct {
  pgb_box box;
  pgb_array4 rY, rY_src, T, rEner, rEner_src, FC, mask;
} pgb_box_view;

/* Counters of the last advance (pgb_reactor_get_stats). hist[b] counts cells whose BDF step
 * count lies in [2^b, 2^(b+1)). nretry counts the cells the mixed-precision pass failed and
 * handed to the FP64 retry pass (gb.retry); nfail counts the cells that failed for good. */
typedef struct {
  unsigned long long ncell, nst, nfe, nje, netf, ncfn, nfail, max_nst;
  unsigned long long hist[16];
  unsigned long long nretry;
} pgb_stats;

/* ReactorBase::create(name) followed by init(reactor_type, ncells)
 * (Source/PeleLM.cpp:706-709). name: "ReactorCvode" (GPU BDF) or "ReactorNull" (forcing only);
 * "ReactorRK64"/"ReactorArkode" are rejected. mechanism: a mechanism compiled into the library
 * (pgb_mechanism_info). reactor_type must be 2 (rho h, constant pressure), the value PeleLM uses.
 * options: whitespace/semicolon separated key=value pairs — the reference's runtime keys
 * ode.rtol, ode.atol, cvode.max_order, cvode.solve_type (dense direct solve with the analytic
 * Jacobian; the GPU decks' matrix-free GMRES / precGMRES keys run that same Newton solve
 * directly), ode.analytical_jacobian,
 * peleLM.use_typ_vals_chem, plus ode.max_steps, gb.precision=fp64|mixed, gb.tpb, gb.graph=0|1,
 * gb.history=shared|global, gb.lu=shared|global, gb.mapping=thread|warp|group (one cell per
 * thread, per warp, or per group of gb.group = 4|8 lanes), gb.wpb, gb.autotune=0|1
 * (time every compiled mapping on the first advance's cells, keep the fastest), gb.retry=0|1
 * (default 1: cells the mixed-precision pass fails are integrated again from their inputs by
 * the FP64 kernel in the same call), and
 * gb.surrogate=<file> (learned surrogate
 * with BDF fallback; no reference counterpart) with threshold overrides gb.sg.audit (audit
 * fraction), gb.sg.mis [K], gb.sg.cons, gb.sg.disT [K], gb.sg.disY, gb.sg.neg,
 * gb.sg.ood_margin, gb.sg.tol_T, gb.sg.tol_Y, gb.sg.models, gb.sg.seed.
 * Returns NULL on error. */
pgb_reactor* pgb_reactor_create(const char* name, const char* mechanism, int reactor_type,
                                const char* options);

/* ReactorBase::set_typ_vals_ode (Source/PeleLM.cpp:1497-1516): n = NUM_SPECIES+1 typical values
 * (rhoY in CGS, then T). With use_typ_vals_chem=1 the absolute tolerance becomes
 * ode.atol * typ[i]. */
int pgb_reactor_set_typ_vals_ode(pgb_reactor* r, const double* typ, int n);

/* ReactorBase::react for one box (Source/PeleLM.cpp:5752): advances every cell of view->box
 * over *dt_react on `stream` (a cudaStream_t, may be NULL) and waits for it. rY, T, rEner and
 * FC are updated in place. *dt_react and *time are left unchanged (the caller resets them,
 * Source/PeleLM.cpp:5759-5760). Returns the number of cells that failed (FC < 0 marks them). */
int pgb_reactor_react(pgb_reactor* r, const pgb_box_view* view, double* dt_react, double* time,
                      void* stream);

/* All boxes of all levels in one persistent launch with a work-stealing cell queue. Stream
 * ordered and asynchronous (returns 0 once enqueued); with gb.graph=1 and a non-default stream
 * the enqueue is captured once per box set into a CUDA graph and replayed. */
int pgb_reactor_react_boxes(pgb_reactor* r, const pgb_box_view* views, int nbox, double dt_react,
                            double time, void* stream);

/* The whole chemistry step of PeleLM::advance_chemistry (Source/PeleLM.cpp:5626-5845) for all
 * boxes in one launch, on the caller's MKS arrays: the MKS -> CGS scaling before react
 * (:5736-5746), the advance, the CGS -> MKS scaling after it (:5763-5771) and the reaction
 * source I_R = -(rhoY_old - rhoY_new) / dt - F_rhoY (:5801) are done inside the kernels' cell
 * load and write-back, so the caller's separate passes and per-box synchronizations go away.
 * rhoY [kg/m^3], rhoH [J/m^3], T [K] in/out; forcing in kg/m^3/s and W/m^3; FC out; mask
 * optional (int, < 0: covered; their state is left untouched); I_R optional (NUM_SPECIES comps,
 * kg/m^3/s; -F for covered cells).
 * Plain BDF and ReactorNull; a reactor with gb.surrogate is refused (it takes CGS arrays). */
typedef struct pgb_chem_view {
  pgb_box box;
  pgb_array4 rhoY, rhoY_src, T, rhoH, rhoH_src, FC, mask, I_R;
} pgb_chem_view;
int pgb_advance_chemistry(pgb_reactor* r, const pgb_chem_view* views, int nbox, double dt, void* stream);

/* Report of the autotuner (reactor created with gb.autotune=1): the time of one advance of a
 * sample of the first call's cells with every compiled BDF mapping and the one kept; empty
 * before the first advance. Returns the report's length. No counterpart in the reference. */
int pgb_reactor_tuning(pgb_reactor* r, char* buf, size_t n);

/* Waits for the last advance on its stream and returns its counters. */
int pgb_reactor_get_stats(pgb_reactor* r, pgb_stats* out);

/* Counters of the learned surrogate in the last advance (reactor created with gb.surrogate).
 * No counterpart in the reference. ncell: unmasked cells; accept: cells written by the
 * surrogate; fallback: cells advanced by the BDF (rejected + audited); ood/mis/cons/ens/neg:
 * cells failing the out-of-distribution, enthalpy, element-conservation, ensemble and
 * negativity checks (a cell may fail several); audit: accepted cells also advanced by the BDF
 * for comparison; audit_bad: audited cells off by more than the audit tolerances; audit_max_*:
 * largest |T| [K] and |Y| differences between surrogate and BDF over the audit sample. */
typedef struct pgb_surrogate_stats {
  unsigned long long ncell, accept, fallback, ood, mis, cons, ens, neg, audit, audit_bad;
  double audit_max_dT, audit_max_dY;
} pgb_surrogate_stats;
int pgb_reactor_get_surrogate_stats(pgb_reactor* r, pgb_surrogate_stats* out);

/* Raw outputs of the reactor's surrogate ensemble for every cell of the boxes (flat cell order),
 * FP32 [cell][member][n_out] in normalised units, through the fused inference kernel; the
 * state is not modified and no gate is applied. in_rows (optional): the network input rows
 * [cell][k_in] (split BF16 features, as FP32). Diagnostics and kernel-vs-training checks; no
 * counterpart in the reference. out, in_rows: device memory. */
int pgb_reactor_surrogate_raw(pgb_reactor* r, const pgb_box_view* views, int nbox, float* out,
                              float* in_rows, void* stream);

/* Surrogate input features of every cell of the boxes (flat cell order, boxes in order, i
 * fastest), FP32, row-major [cell][2 NS + 2]: log10 max(Y_k, 1e-14), T, F_rhoY_k / rho,
 * F_rhoh / rho; masked cells get zeros. The same device code the inference kernel uses, so
 * training sets see the kernel's bits. out: device memory. No counterpart in the reference. */
int pgb_surrogate_features(const char* mechanism, const pgb_box_view* views, int nbox, float* out,
                           void* stream);

/* ReactorBase::close (Source/PeleLM.cpp:930) and destruction. */
void pgb_reactor_close(pgb_reactor* r);

/* Copies the last error message of the calling thread; returns its length. */
int pgb_last_error(char* buf, size_t n);

/* Species / reaction counts of a compiled mechanism; returns 0 if known, -1 otherwise. */
int pgb_mechanism_info(const char* mechanism, int* nspecies, int* nreactions);

/* Library identification (ABI version, build arch). */
int pgb_version(void);

/* Instantaneous production rates, the per-cell work of reactionRateRhoY
 * (Source/PeleLM_K.H:54-98) called from compute_instantaneous_reaction_rates
 * (Source/PeleLM.cpp:2013-2074). MKS in and out, as there: rhoY (kg/m^3), rhoH (J/m^3), T (K,
 * initial guess, refined by HY2T), mask; writes rhoYdot (kg/m^3/s). The view's rY_src / rEner_src
 * / FC fields are unused; rhoYdot goes to `out`. */
int pgb_reaction_rates(const char* mechanism, const pgb_box_view* view, const pgb_array4* out,
                       void* stream);

/* Heat release rate HR = -sum_k rhoYdot_k h_k(T) [W/m^3]: the HeatRelease derive
 * (Source/PeleLM_derive.cpp:627-650, registered at Source/PeleLM_setup.cpp:838-840). MKS in:
 * T [K] (1 comp), rhoYdot [kg/m^3/s] (NUM_SPECIES comps, the reaction source I_R); out: hr
 * (1 comp). Arrays must cover the box. */
int pgb_heat_release(const char* mechanism, const pgb_box* box, const pgb_array4* T,
                     const pgb_array4* rhoYdot, const pgb_array4* hr, void* stream);

/* Diagnostic: the Newton matrix pieces of the BDF kernels for ncell states, so a test can
 * compare them with an independent implementation. No counterpart in the reference (inside it
 * these are CVODE's Jacobian and dense linear solve, cvode.solve_type = denseAJ_direct,
 * Exec/RegTests/FlameSheet/inputs.2d-regt:86-91). mapping 1: the warp and lane-group kernels
 * (J and x); mapping 0: the cell-per-thread kernels (J only, x set to NaN; an error for
 * mechanisms compiled without them). Device arrays, cell-major, CGS: y [ncell][N] (rhoY, then T;
 * N = NUM_SPECIES + 1), F [ncell][NUM_SPECIES] rhoY forcing, Fh [ncell] rho h forcing, b
 * [ncell][N]. Out: J [ncell][N][N] row-major (d ydot_i / d y_k, the analytic Jacobian the
 * kernels build), x [ncell][N] solving (I - gamma J) x = b through their partial-pivot LU and
 * triangular solves (NaN where the matrix is singular). fp64 = 0 runs the FP32 Jacobian and LU
 * of mixed precision. Stream ordered. */
int pgb_newton_matrix(const char* mechanism, int mapping, long long ncell, const double* y,
                      const double* F, const double* Fh, double gamma, const double* b, int fp64,
                      double* J, double* x, void* stream);

/* T from (rho h, Y): the per-cell work of RhoH_to_Temp / getTfromHY (Source/PeleLM.cpp:8201-8287,
 * Source/PeleLM_K.H:508-529). MKS in: rhoY (view->rY), rhoH (view->rEner), T in/out (view->T).
 * Newton iteration clipped to [tmin, tmax]. */
int pgb_rhoh_to_temp(const char* mechanism, const pgb_box_view* view, double tmin, double tmax,
                     void* stream);

/* Allocation-free advance of up to PGB_NOALLOC_MAX_BOXES boxes, for callers that cannot
 * allocate device memory at react time. No counterpart in the reference. PeleLM, for example,
 * runs on an AMReX arena that reserves most of the GPU at start-up, so a cudaMalloc issued by
 * the reactor in the middle of a time step can fail or fragment what the arena left, and
 * cudaMalloc/cudaFree can synchronize the device. This entry point allocates nothing — no
 * cudaMalloc, cudaFree or other allocating routine: the caller passes all inputs and outputs
 * through the box views, and the scratch (box table, work-queue head, counters) is one fixed
 * device array inside the library, about 370 KB, which every GPU that loads the library holds
 * until the process exits. It runs the persistent work-stealing kernels of
 * pgb_reactor_react_boxes with their working state in shared memory — cell per thread for the
 * 9-species mechanism, cell per warp for the larger ones — with cvode.max_order = max_order,
 * ode.max_steps = max_steps and FP64 (fp64 != 0) or mixed (fp64 == 0) Jacobian precision.
 * The tolerances are uniform: rtol, and atol on every component. The typical-value scaling of
 * set_typ_vals_ode / peleLM.use_typ_vals_chem does not apply here (there is no reactor object
 * to hold the typical values), so results equal those of a reactor created without it.
 * - nbox must be in [1, PGB_NOALLOC_MAX_BOXES]; larger box lists are rejected with an error.
 * - The first call on a device (with that device current) resolves the scratch array's device
 *   address; make that first call before any stream capture.
 * - Capturable: the box table reaches the scratch array through kernel parameters (no host
 *   buffer outlives the call), so a captured call replays with the views it was captured with.
 *   stats must be NULL while the stream is capturing (they wait for the advance); the call
 *   returns an error otherwise.
 * - All calls on a device share the one scratch array, which keeps the last call's contents
 *   (the queue head and counters are cleared on each call). Calls whose work overlaps on the
 *   GPU — concurrent streams or threads — race on it: serialize them.
 * - Stream ordered; if stats is non-NULL the call waits for the advance and fills it.
 * - No FP64 retry pass (it would need a failed-cell list sized by the cell count): a cell that
 *   fails keeps its state at failure and FC = -status, as with gb.retry=0.
 * Returns 0 on success, -1 on error (pgb_last_error). */
#define PGB_NOALLOC_MAX_BOXES 1024
int pgb_react_boxes_noalloc(const char* mechanism, const pgb_box_view* views, int nbox,
                            double dt_react, double rtol, double atol, int max_order, int max_steps,
                            int fp64, void* stream, pgb_stats* stats);

/* ---- Work partition across ranks (one rank per GPU); host-only, no device call. ----
 * The analogue of PeleLM's chemistry load balance on CPU builds: chop the grids until there are
 * enough boxes per rank (Source/PeleLM.cpp:5699-5723), then a knapsack over each box's summed
 * FuncCount of the previous advance (getFuncCountDM, Source/PeleLM.cpp:5530-5623). The cells are
 * independent, so each rank advances its boxes with no communication. */

/* Halves the longest side of the largest box (ties: first) while the list holds fewer than
 * `target` boxes and a box has a side of at least 2 * min_side; each piece keeps its parent's
 * index in parent[] (the caller's arrays still cover it). out/parent hold `cap` entries.
 * Returns the number of boxes written, or -1. */
int pgb_chop_boxes(const pgb_box* in, int nin, int min_side, int target, pgb_box* out, int* parent, int cap);

/* Assigns box b (weight[b] >= 0: its FC sum, or its cell count before the first advance) to
 * rank_of_box[b] in [0, nranks): heaviest first to the least loaded rank, then moves and swaps
 * between the most and least loaded ranks while the largest load strictly drops. Deterministic.
 * load (optional, nranks entries) receives each rank's total. The largest load is at most the
 * mean load plus the largest weight. Returns 0, or -1. */
int pgb_partition_boxes(const double* weight, int nbox, int nranks, int* rank_of_box, double* load);

/* ---- Learned surrogate: BF16 tensor-core building blocks (FP32 accumulation). No counterpart in
 * the reference: they train and evaluate the MLP that predicts a cell's (dY, dT) over dt_react.
 * All pointers are device memory; bf16 arrays are passed as void*. ---- */

/* C[m][n] = act(sum_k A[m][k] B[n][k] + bias[n]); A (M x K, lda), B (N x K, ldb) row-major BF16;
 * K % 32 == 0. Writes the FP32 pre-activation to `pre`, and/or the result as BF16 (`out_bf16`) /
 * FP32 (`out_f32`), all with leading dimension ldo; columns >= n_valid are written as 0.
 * act: 0 identity, 1 GELU (tanh form). */
int pgb_mlp_gemm_nt(const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                    const float* bias, int act, float* pre, void* out_bf16, float* out_f32, int ldo,
                    int n_valid, void* stream);
/* out (cols x rows, ldo) = in^T (rows x cols, ldi), BF16. */
int pgb_mlp_transpose_bf16(const void* in, int rows, int cols, int ldi, void* out, int ldo, void* stream);
/* dZ = dA * GELU'(pre), n elements (BF16 out, optional FP32 copy dZf). */
int pgb_mlp_gelu_backward(const float* dA, const float* pre, void* dZ, float* dZf, long long n, void* stream);
/* MSE over the first n_valid of ld columns: dY = 2 (Y - T) / (M n_valid) (FP32 and BF16), *loss += sum d^2. */
int pgb_mlp_mse_grad(const float* Y, const float* T, int M, int ld, int n_valid, float* dYf, void* dY,
                     float* loss, void* stream);
/* db[n] = sum_m dZ[m][n]. */
int pgb_mlp_bias_grad(const float* dZ, int M, int N, int ld, float* db, void* stream);
/* Adam step `step` (>= 1) on FP32 parameters p with moments m, v; refreshes the BF16 copy p_bf16. */
int pgb_mlp_adam(float* p, const float* g, float* m, float* v, void* p_bf16, long long n, float lr,
                 float b1, float b2, float eps, int step, void* stream);
int pgb_mlp_f32_to_bf16(const float* in, void* out, long long n, void* stream);
/* First-layer weight for a split input: each FP32 row of W (rows x cols) is written to out
 * (row stride ldo >= 2*cols) twice as BF16, at columns [0, cols) and [cols, 2*cols). */
int pgb_mlp_dup_weight_bf16(const float* W, int rows, int cols, void* out, int ldo, void* stream);
/* Splits FP32 rows x (row stride ldx) into BF16 high parts at out columns [0, cols) and BF16
 * low parts (x - high) at columns [off, off + cols); row stride of out is ldo. */
int pgb_mlp_split_rows_bf16(const float* x, int rows, int cols, int ldx, void* out, int ldo, int off,
                            void* stream);

/* Measures the device's FP64 FMA throughput in TFLOP/s (2 flops per FMA). No counterpart in
 * the reference: a measurement utility giving the roofline denominator of the FP64-bound
 * reactor kernels. */
int pgb_fp64_peak_tflops(int iters, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* PELELM_GB300_H */
