/*
 * sclet_gb300 -- C ABI of the GB300 (sm_103a) implementation of the ScLETD
 * exponential-time-differencing step (beta->omega / beta->alpha phase field).
 *
 * The reference keeps its state in process globals and exits on error; this
 * boundary keeps the same step sequence and file formats behind an opaque
 * context that owns the device-resident state, and returns an int status
 * (SCLET_OK = 0) instead of calling exit().  Plain pointers and sizes only.
 *
 * Each entry point names the reference routine it replaces
 * (paths relative to the reference project).
 *
 * Field blocks are n*n*n doubles (n = N + 4: N owned cells plus two ghost
 * layers per side), index z*n*n + y*n + x, exactly the reference's
 * ac[m].fieldE / ch[m].fieldCI layout (source_beta_to_omega/src/ScLETD.h:60-96).
 * Field kinds: SCLET_AC (non-conserved order parameters eta_m, m < nac) and
 * SCLET_CH (conserved concentrations c_m, m < nch).
 */
#ifndef SCLET_GB300_H
#define SCLET_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SCLET_OK 0
#define SCLET_ERR_ARG 1         /* bad argument or unsupported size          */
#define SCLET_ERR_IO 2          /* input file missing or malformed           */
#define SCLET_ERR_CUDA 3        /* CUDA runtime error (message: last_error)  */
#define SCLET_ERR_UNSUPPORTED 4 /* option the reference path does not take   */
#define SCLET_ERR_NOMEM 5       /* device allocation failed                  */
#define SCLET_ERR_TIMEOUT 6     /* a bounded device wait gave up             */
#define SCLET_ERR_NONFINITE 7   /* a diagnostic found NaN/Inf in the state   */

#define SCLET_AC 0
#define SCLET_CH 1

/* Arithmetic of the step.  SCLET_FP64: every stage in FP64 (the plain form,
 * checked against the reference).  SCLET_MIXED: eigenbasis products as
 * split-precision tensor-core products with FP32 accumulation, stencils and
 * FFT in FP32, diagnostics and mass correction in FP64. */
#define SCLET_FP64 0
#define SCLET_MIXED 1

/* Physics plugins (sclet_params.physics), the drop-in replacements of the
 * reference's formula.c (init_KL, AC_f, CH_f; source_beta_to_omega/src/
 * formula.c:9-56), each one source compiled for the host and the device
 * (energy-stability_gb300/plugins/):
 *   SCLET_PHYSICS_LANDAU246  Landau 2-4-6 with cross term and c-eta coupling,
 *                            constants from landau_input.txt (landau[])
 *   SCLET_PHYSICS_FORMULA234 the reference's own formula.c: LE = 1, KE = 42,
 *                            the 2-3-4 polynomial; order parameters only */
#define SCLET_PHYSICS_LANDAU246 0
#define SCLET_PHYSICS_FORMULA234 1

typedef struct sclet_ctx sclet_ctx;

/* Everything the reference reads from its input files. */
typedef struct sclet_params {
  /* input<suffix>.ini, positional (source_beta_to_omega/src/ScLETD.c:16-34) */
  int nx, ny, nz;          /* local block incl. ghosts; must be equal here   */
  int px, py, pz;          /* process grid; 1,1,1 on one GPU                 */
  int nghost;              /* 2                                              */
  char work_dir[1024];
  char data_dir[1024];
  double dt, t_total;
  double epn2;
  int periodic;            /* 1                                              */
  int nac, nch;
  int restart, restart_iter;
  char restart_dir[1024];
  double xmin, ymin, zmin, xmax, ymax, zmax;
  int etd2;                /* 1: second-order corrector                      */
  int elastic;             /* 0 none, 1 elastic force on the AC fields       */
  int anisotropic;         /* 1: explicit div(lambda grad eta) term          */
  double kkx, kky, kkz;
  int variable_mobility;   /* 0 constant mobility; 1 variable mobility       */
                           /* (mobility.c:838-922: nch = 1, nac >= 1)        */
  /* elastic_input.txt (source_beta_to_omega/src/elastic.c:349-439) */
  double elastic_scale;
  double voigt[36];        /* 6x6, order 11,22,33,23,13,12                   */
  double eigenstrain[4][9];
  /* anisotropic_input.txt (source_beta_to_omega/src/anisotropic.c:630-674):
   * the file tensors; the step uses diag(kk) - lambda_file */
  double lambda_file[4][9];
  /* physics plugin constants (replaces the compile-time constants of
   * source_beta_to_omega/src/formula.c:9-38): a2 a4 a6 g th c0 A LE KE LCI KCI
   * for SCLET_PHYSICS_LANDAU246 */
  double landau[11];
  /* which physics plugin (SCLET_PHYSICS_*); the reference selects its
   * formula.c at link time.  Default SCLET_PHYSICS_LANDAU246. */
  int physics;
} sclet_params;

/* Diagnostics of one state (check_soln_new, field.c:407-678), per field. */
typedef struct sclet_diag {
  double max, min, vol, energy;
} sclet_diag;

/* ---- input files (host only; no GPU needed) ---------------------------- */
/* Defaults of the 64^3 beta->omega case; all file readers start from them. */
void sclet_params_default(sclet_params *p);
/* main()'s ini parse, ScLETD.c:16-34 */
int sclet_read_ini(const char *path, sclet_params *p);
/* elastic_input(), elastic.c:349-439 */
int sclet_read_elastic_input(const char *path, sclet_params *p);
/* anisotropic_input(), anisotropic.c:630-674 (file tensors only) */
int sclet_read_anisotropic_input(const char *path, sclet_params *p);
/* init_KL() constants of the physics plugin (formula.c:9-19); 11 numbers */
int sclet_read_landau_input(const char *path, sclet_params *p);
/* All of the above from a run directory, as main() does (ScLETD.c:15-72);
 * landau_input.txt and physics_input.txt (one word: the plugin name,
 * "landau246" or "formula234") are optional.  The reference picks its
 * formula.c when it is built; physics_input.txt is this library's stand-in. */
int sclet_read_case(const char *dir, const char *suffix, sclet_params *p);
/* One eigen variant as read_matrices() reads it (vars.c:370-476):
 * d<k><n>.dat (n values), v<k><n>.dat and vi<k><n>.dat (n x n, row by row).
 * d, v, vi receive n, n*n, n*n doubles; v and vi row-major. */
int sclet_read_eigen(const char *dir, int n, int variant, double *d, double *v, double *vi);
/* Closed-form Dirichlet-Dirichlet basis (variant 3, the one a periodic single
 * block selects in read_matrices, vars.c:488-582): the DST-I, eigenvalues
 * ascending, v = vi^T = vi.  Same output layout as sclet_read_eigen. */
void sclet_eigen_dirichlet(int n, double *d, double *v, double *vi);
/* Seeded initial value of cell (x, y, z) of field f, uniform in [lo, hi):
 * SplitMix64 on (seed, field, owned-cell index z*N*N + y*N + x). */
double sclet_seeded_value(unsigned long long seed, int field, long long cell, double lo, double hi);
/* Writes the interior of a field block as restart text (write_field,
 * field.c:156-174) / reads it (read_field, field.c:137-154). */
int sclet_write_restart(const char *path, int n, const double *block);
int sclet_read_restart(const char *path, int n, double *block);
/* Checkpoint files of the alpha driver (source_beta_to_alpha/src/vars.c):
 * write_chk (:966-989) writes, per order parameter, the step counter as one
 * int and then every cell of the n^3 block, ghost layers included, as
 * doubles in native byte order; read_chk (:1012-1035) reads them back (a
 * short file is an error here).  File names: sclet_chk_path gives
 * "<dir>00/eta<m>_chk<chk>_000000.dat" (rank (0, 0, 0) of one block, the
 * rank's z coordinate naming the sub-directory, vars.c:975), and
 * sclet_field2b_path gives "<dir>00/eta<m>_<irun:06d>_000000.dat" (or
 * "c<m>_..." for a concentration) for the 16-bit files (vars.c:1079). */
int sclet_write_chk_file(const char *path, int irun, int n, const double *block);
int sclet_read_chk_file(const char *path, int n, int *irun, double *block);
int sclet_chk_path(char *out, size_t len, const char *dir, int m, int chk);
int sclet_field2b_path(char *out, size_t len, const char *dir, int kind, int m, int irun);
/* Plain-text VTK of nfields blocks (visualisation/write_vtk.py): a legacy
 * ASCII structured grid of the whole n^3 block, points with x fastest written
 * as (z, y, x), one float scalar block "eta<m>" per field, values in %14.6e. */
int sclet_write_vtk_file(const char *path, int istep, int n, int nfields, const double *blocks);

/* ---- context ----------------------------------------------------------- */
/* alloc_vars (vars.c:166-300), init_para (vars.c:58-157), read_matrices
 * (vars.c:361-591; closed-form variant 3 unless sclet_set_eigen is called),
 * ac_init_phi/ch_init_phi (vars.c:302-359) and elastic_init (elastic.c:607)
 * on device `device`.  Fields start at zero. */
int sclet_create(const sclet_params *p, int precision, int device, sclet_ctx **out);
/* No counterpart in the reference (one run per process there): `runs`
 * independent runs of the same parameters and block size side by side in one
 * context (the batched ensemble), each with its own state and, when krun is
 * not NULL, its own value krun[r] of plugin constant 0 (the Landau a2).
 * Every stage is one launch over all runs.  Run r's fields are the blocks
 * r F .. r F + F - 1 of the host arrays of sclet_set_fields /
 * sclet_get_fields, and of sclet_check_soln's output; sclet_field_count gives
 * runs F.  runs > 1 needs SCLET_MIXED and nch = 0; per-field accessors then
 * return SCLET_ERR_UNSUPPORTED. */
int sclet_create_runs(const sclet_params *p, int runs, const double *krun, int precision, int device,
                      sclet_ctx **out);
/* dealloc_vars (vars.c:593-732), elastic_finish (elastic.c:276-300) */
void sclet_destroy(sclet_ctx *ctx);
/* Last error message of this context (or of the last failed create). */
const char *sclet_last_error(const sclet_ctx *ctx);
/* Replaces the per-axis eigen data (all three axes use the same n-point
 * basis, as read_matrices does for nx = ny = nz): d (n, unscaled; divided by
 * h^2 here as vars.c:512 does), v and vi row-major n x n. */
int sclet_set_eigen(sclet_ctx *ctx, const double *d, const double *v, const double *vi);
/* Block edge n, field count (of every run), and the CUDA stream the context
 * runs on. */
int sclet_block_edge(const sclet_ctx *ctx);
int sclet_field_count(const sclet_ctx *ctx);
void *sclet_stream(const sclet_ctx *ctx);

/* ---- state transfer (host <-> device) ---------------------------------- */
int sclet_set_field(sclet_ctx *ctx, int kind, int m, const double *block);
int sclet_get_field(sclet_ctx *ctx, int kind, int m, double *block);
/* No counterpart in the reference, whose fields live in host memory.  All
 * fields at once: host holds field-count blocks of n^3 doubles, AC fields
 * first.  sclet_set_fields returns when the state holds them;
 * sclet_get_fields when host holds the state. */
int sclet_set_fields(sclet_ctx *ctx, const double *host);
int sclet_get_fields(sclet_ctx *ctx, double *host);
/* Pipelined forms: the copies run on copy engines on one stream per direction
 * (overlapping the steps when host is page-locked, sclet_host_alloc) through
 * an FP64 staging area per direction, allocated on first use.  In the
 * context's stream order, set_fields_async replaces the state and
 * get_fields_async reads it, so a caller may queue
 *   set(step k+1 inputs) while step k runs, and get(step k results) before it;
 * host must stay valid and unchanged (set) or unread (get) until sclet_sync
 * returns, which waits for both copy streams too. */
int sclet_set_fields_async(sclet_ctx *ctx, const double *host);
int sclet_get_fields_async(sclet_ctx *ctx, double *host);
/* init_field with restart = 1 (field.c:743-755): interior from text. */
int sclet_load_restart(sclet_ctx *ctx, int kind, int m, const char *path);

/* ---- step routines (the reference's time-loop pieces) ------------------ */
/* transfer(), trans.c:1939-1996: ghost exchange of every field. */
int sclet_transfer(sclet_ctx *ctx);
/* elastic_calculate(), elastic.c:689-763 (ELASTIC == 1). */
int sclet_elastic_calculate(sclet_ctx *ctx);
/* calc_mu() + ac_calc_FU / ch_calc_FU for every field (trans.c:1998-2013,
 * calc.c:8-68, 70-487) into slot 1 (fieldE1/fieldCI1) or 2 (fieldE2/...). */
int sclet_calc_rhs(sclet_ctx *ctx, int slot);
/* PUX/PUY/PUZ + ac_updateU_new/ch_updateU_new + zxy_xyz + back transform for
 * every field (ScLETD.c:105-142, calc.c:489-535, 585-684). */
int sclet_etd_update(sclet_ctx *ctx);
/* ETD2 corrector: prepare_U1_new .. correct_U_new (ScLETD.c:159-188,
 * calc.c:537-583), after transfer/elastic/calc_rhs(slot 2). */
int sclet_etd2_correct(sclet_ctx *ctx);
/* `nsteps` passes of the time-loop body (ScLETD.c:86-190), asynchronous on
 * the context's stream. */
int sclet_step(sclet_ctx *ctx, int nsteps);
/* check_soln_new(), field.c:407-678: diagnostics of the current state
 * (compensated FP64 reduction on the device; out has field-count entries,
 * AC fields first).  energy_form 0: the reference's hard-coded polynomial and
 * its per-kind energies; 1: the plugin's total free energy. */
int sclet_check_soln(sclet_ctx *ctx, int energy_form, sclet_diag *out);
/* The reference's loop runs check_soln_new after every pass (ScLETD.c:86-190).
 * With energy_form 0 or 1, sclet_step queues the same reductions after each
 * step on the context's stream (no host synchronisation); -1 (the default)
 * queues none.  sclet_last_diagnostics waits for the stream and returns the
 * most recent record. */
int sclet_set_step_diagnostics(sclet_ctx *ctx, int energy_form);
int sclet_last_diagnostics(sclet_ctx *ctx, sclet_diag *out);
/* Gradient tensors used by the energy (per AC field, 3x3 row-major).  The
 * default is the gradient operator of the dynamics: lambda_file when
 * anisotropic, else diag(kk). */
int sclet_set_energy_tensors(sclet_ctx *ctx, const double *lam /* nac*9 */);
/* The log files of check_soln_new (field.c:419-455, 524, 591, 647): under
 * work_dir, one row "iter,max,min,vol,eng" (%+1.15f) per field appended to
 * phi_ac_<m>.csv / phi_ch_<m>.csv, and "iter,eng" to phi_couple.csv when
 * couple is non-NULL and both kinds are present; iter 0 starts each file with
 * the reference's header line.  d has nac + nch entries, AC fields first. */
int sclet_append_soln_log(const char *work_dir, int iter, int nac, int nch, const sclet_diag *d, const double *couple);
/* sclet_check_soln(energy_form) of the context written as those logs; the
 * coupled energy is the plugin's total free energy (energy_form 1).  The
 * reference's coupled sum takes the gradients of the first nch AC fields
 * only (field.c:608-636); here it takes all of them, as the energy the
 * scheme decreases. */
int sclet_log_soln(sclet_ctx *ctx, const char *work_dir, int iter, int energy_form);

/* ---- checkpoint and 16-bit output files (the alpha driver's formats) ---- */
/* write_chk / read_chk (source_beta_to_alpha/src/vars.c:966-1035) for every
 * order parameter of the context, under dir (the reference's work_dir; the
 * rank sub-directory "00" is created when missing).  The reference's
 * concentration checkpoints are compiled out (vars.c:990-1010), so are these. */
int sclet_write_chk(sclet_ctx *ctx, const char *dir, int chk, int irun);
int sclet_read_chk(sclet_ctx *ctx, const char *dir, int chk, int *irun);
/* Dtype2B_E / Dtype2B_CI (anisotropic_hip.c:3920-3944): the 16-bit code of
 * every cell of one field's n^3 block into out (n^3 host values): order
 * parameters (eta + 0.1) * 30000, concentrations c * 50000, computed in FP64
 * and truncated toward zero.  The reference's conversion is undefined outside
 * [0, 65535]; these codes saturate there. */
int sclet_field_u16(sclet_ctx *ctx, int kind, int m, unsigned short *out);
/* write_field2B (vars.c:1066-1116): the codes of every order parameter
 * (mode 0) or concentration (mode 1) as raw 16-bit files under data_dir. */
int sclet_write_field2b(sclet_ctx *ctx, const char *data_dir, int irun, int mode);
/* The order parameters of the context as one VTK file (sclet_write_vtk_file). */
int sclet_write_vtk(sclet_ctx *ctx, const char *path, int istep);

/* ---- inspection (host buffers) ------------------------------------------ */
/* fieldE1/fieldE2 of one field, and the elastic force felas.  In the mixed
 * form the conserved field is held as c - c0, and its right-hand side is that
 * of c minus that of the constant state c0 (zero away from the block faces). */
int sclet_get_rhs(sclet_ctx *ctx, int slot, int kind, int m, double *block);
int sclet_get_felas(sclet_ctx *ctx, int m, double *block);
/* One mode-n product with layout rotation (one PUX/PUY/PUZ contraction,
 * calc.c:631-684): out[b + n*c + n*n*a'] = sum_a M(a', a) in[a + n*b + n*n*c]
 * with M = V^-1 (inverse = 0) or V (inverse = 1) of axis 0. */
int sclet_mode_product(sclet_ctx *ctx, int inverse, const double *in, double *out);

/* ---- synchronisation and timing ---------------------------------------- */
/* Waits for the context's work; SCLET_ERR_TIMEOUT when a bounded device wait
 * gave up since the last call (reported once, then cleared). */
int sclet_sync(sclet_ctx *ctx);
/* Runs `nsteps` steps between two CUDA events on the context's stream and
 * returns the elapsed milliseconds. */
int sclet_time_steps(sclet_ctx *ctx, int nsteps, float *ms);
/* Per-kernel-class timing of the last sclet_time_steps call when profiling
 * was enabled with sclet_set_profiling(ctx, 1): ms[k] for classes
 * 0 mode-n products (all of the eigenbasis transforms and the update),
 * 1 right-hand sides, 2 FFT/elastic, 3 halo, 4 diagnostics, and within class
 * 0 of the mixed form: 5 tensor-core product kernels, 6 slicing kernels;
 * launches[k] kernel launches.  Up to 8 classes. */
int sclet_set_profiling(sclet_ctx *ctx, int on);
int sclet_stage_times(const sclet_ctx *ctx, float *ms, int *launches, int nclasses);
/* No counterpart in the reference.  sclet_step's work captured once as a
 * CUDA graph (on the first call; a context that has not stepped yet takes
 * its first step uncaptured) and replayed nsteps times on the context's
 * stream: the same launches with the host's launch cost paid once. */
int sclet_graph_step(sclet_ctx *ctx, int nsteps);
/* No counterpart in the reference.  Autotuner of the mixed form's launch
 * shapes: times `trials` steps of each candidate (z-planes per CTA of the
 * Allen-Cahn right-hand side: 8, 16, 32, 64; then persistent CTAs of the
 * tensor-core products: all SMs, 3/4, 1/2), keeps the fastest and puts the
 * state back after every trial, so results do not change.  choice (2 ints,
 * may be NULL) receives the z-planes and the CTA count (0: all SMs). */
int sclet_tune(sclet_ctx *ctx, int trials, int *choice);
/* The batched ensemble (no counterpart in the reference): contexts of
 * several block sizes (each holding its runs side by side) advanced
 * together; sclet_ensemble_step captures one step of all of them as one
 * CUDA graph, one branch per context on the context's stream, and replays
 * it (contexts that have not stepped yet take one uncaptured step first).
 * The contexts stay owned by the caller and must outlive the ensemble. */
typedef struct sclet_ensemble sclet_ensemble;
int sclet_ensemble_create(sclet_ctx *const *ctxs, int count, sclet_ensemble **out);
void sclet_ensemble_destroy(sclet_ensemble *e);
const char *sclet_ensemble_last_error(const sclet_ensemble *e);
int sclet_ensemble_step(sclet_ensemble *e, int nsteps);
int sclet_ensemble_sync(sclet_ensemble *e);
/* nsteps ensemble steps between two CUDA events; elapsed milliseconds. */
int sclet_ensemble_time_steps(sclet_ensemble *e, int nsteps, float *ms);
/* No counterpart in the reference.  Self-test of the bounded device waits
 * (mixed form): one tensor-core product launch whose producer issues no
 * loads, so its MMA and epilogue warps wait on barriers that nothing arrives
 * on until their poll limit (about half a second), then record the error, free
 * their tensor memory and return.  Returns what sclet_sync reports:
 * SCLET_ERR_TIMEOUT when the waits gave up as they must; the error is then
 * cleared and the context stays usable (the state is not touched). */
int sclet_selftest_wait_timeout(sclet_ctx *ctx);
/* No counterpart in the reference.  The device's FP64 fused multiply-add
 * rate in TFLOP/s (eight independent chains per thread on every SM, best of
 * three timed launches): the roofline of the plain form's FP64-bound stages. */
int sclet_measure_fp64_rate(int device, double *tflops);
/* Kernel launches issued by this context so far. */
long long sclet_launch_count(const sclet_ctx *ctx);
/* Page-locked host buffers for the field blocks (no reference counterpart:
 * the reference's arrays are plain host memory, vars.c:166-300).  Copies
 * from/to these overlap nothing else but run at full link speed. */
void *sclet_host_alloc(size_t bytes);
void sclet_host_free(void *ptr);

/* ---- diagnostics without allocation ------------------------------------- */
/* No counterpart in the reference, whose check_soln_new (field.c:407-678)
 * reads the process-global arrays.  The same diagnostics as sclet_check_soln
 * (same kernels, default gradient tensors) of a state block the caller holds
 * on the current device, for callers that must not allocate: a fixed memory
 * budget or pool, or work already queued on other streams that a cudaMalloc
 * would stall.  It allocates nothing and needs no context: scratch is a fixed
 * device array inside the library (about 230 KB per device).
 *   fields    device, field-count blocks of nx^3 cells, AC fields first:
 *             double when precision = SCLET_FP64, float when SCLET_MIXED
 *   out       device, 4 doubles per field: max, min, vol, energy
 *   stream    cudaStream_t on the current device (NULL: legacy default)
 *   msg       optional buffer for the error text (msg_len bytes)
 * Returns after queuing the work (SCLET_OK) or an error code; more than
 * SCLET_NOALLOC_MAX_FIELDS fields is SCLET_ERR_ARG.  The first call on a
 * device looks the scratch address up (set-up); make it before any stream
 * capture.  The scratch is shared: calls that overlap in time on one device
 * race on it, so order them on one stream. */
#define SCLET_NOALLOC_MAX_FIELDS 5
int sclet_check_soln_noalloc(const sclet_params *p, int precision, const void *fields, int energy_form,
                             double *out, void *stream, char *msg, size_t msg_len);

/* ---- learned coarse-step corrector --------------------------------------- */
/* No counterpart in the reference (its CNN, source_beta_to_alpha/src/CNN.cpp,
 * is an unrelated detector).  A 3-D residual convolution network (3x3x3
 * periodic kernels, SCLET_NET_WIDTH channels, SCLET_NET_BLOCKS residual
 * blocks of two convolutions, ReLU; BF16 weights and activations, FP32
 * accumulation, FP32 master weights and Adam) that maps (coarse ETD state,
 * start state) to a correction of the coarse state toward the state after
 * the fine steps it replaces.  Forward and backward run on the project's own
 * kernels (tcgen05 implicit-GEMM convolutions).  Device arrays are FP32
 * planar over the owned cells: in [batch][SCLET_NET_IN][N^3], out / target
 * [batch][SCLET_NET_OUT][N^3]; N a periodic grid edge >= 4.  As the learned
 * step uses it, in holds the start state u0 and the coarse increment
 * D = coarse(u0) - u0 divided by the scale s = RMS(D) + SCLET_NET_FLOOR RMS(u0)
 * (RMS over every cell and field), and s out is the correction of the coarse
 * state. */
#define SCLET_NET_FLOOR 1e-3
#define SCLET_NET_IN 8
#define SCLET_NET_OUT 4
#define SCLET_NET_WIDTH 32
#define SCLET_NET_BLOCKS 4
typedef struct sclet_net sclet_net;
/* Deterministic initial parameters from seed; out_scale multiplies the
 * output (the correction starts at zero: the output layer is zero). */
int sclet_net_create(int device, unsigned long long seed, float out_scale, sclet_net **out);
void sclet_net_destroy(sclet_net *net);
const char *sclet_net_last_error(const sclet_net *net);
void *sclet_net_stream(const sclet_net *net);
/* FP32 parameters: weights [layer][27 taps][32 out][32 in] (taps
 * t = 9 (dz+1) + 3 (dy+1) + (dx+1); unused input/output channels zero), then
 * biases [layer][32], for 2 + 2 SCLET_NET_BLOCKS layers. */
long long sclet_net_param_count(void);
int sclet_net_get_params(sclet_net *net, float *host);
int sclet_net_set_params(sclet_net *net, const float *host);
/* out = net(in), queued on the network's stream (sclet_net_sync waits). */
int sclet_net_forward(sclet_net *net, int N, int batch, const float *in, float *out);
int sclet_net_sync(sclet_net *net);
/* loss = mean of (net(in) - target)^2 over every value, and the gradient of
 * every parameter (grad_host: sclet_net_param_count floats, may be NULL).
 * Synchronous. */
int sclet_net_gradient(sclet_net *net, int N, int batch, const float *in, const float *target, double *loss,
                       float *grad_host);
/* sclet_net_gradient followed by one Adam step (beta 0.9 / 0.999). */
int sclet_net_train_step(sclet_net *net, int N, int batch, const float *in, const float *target, float lr,
                         double *loss);
/* Input runs of the convolution kernel per 128-cell tile, process-wide: 0
 * chooses by N (the default), 1 one run per stencil plane and channel chunk,
 * 3 one run per stencil row.  Both tilings compute the same sums in the same
 * order; the setting is there to test that.  Returns the previous setting,
 * or -1 for a value other than 0, 1, 3. */
int sclet_net_set_conv_runs(int runs_per_plane);

/* Coarse steps judged by the plain-ETD checks.  coarse and fine are two
 * contexts of the same run on one device, coarse.dt = ratio * fine.dt.  Each
 * of nsteps steps: one ETD step of coarse from state u0 (the coarse
 * context's state), corrected by the network when net is not NULL (input u0
 * and the increment over the scale s, correction s times the output); then
 *   energy:    the free energy (check_soln_new, the plugin's total form) must
 *              not exceed that of u0 by more than energy_tol relative;
 *   mass:      each conserved field's integral must equal u0's to 1e-10
 *              relative (the correction of a conserved field has its mean
 *              removed, so this holds up to the FP32 rounding of the state);
 *   deviation: every check_every steps (0: never) the fine context runs ratio
 *              steps from u0, and the per-field relative L2 distance of the
 *              step's result from it must not exceed deviation_bound.
 * A step that fails any check is replaced by ratio fine steps from u0
 * (the fallback).  The coarse context holds the accepted state after each
 * step.  Counters accumulate into st. */
typedef struct sclet_learned_stats {
  long long steps, fallbacks, energy_fail, mass_fail, deviation_fail, deviation_checks;
  double max_deviation;
} sclet_learned_stats;
int sclet_learned_step(sclet_ctx *coarse, sclet_ctx *fine, sclet_net *net, int ratio, int nsteps, int check_every,
                       double deviation_bound, double energy_tol, sclet_learned_stats *st);

#ifdef __cplusplus
}
#endif
#endif
