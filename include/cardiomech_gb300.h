/* cardiomech_gb300.h -- C ABI of the GB300 cell-model update library (libcmgb300.so).
 *
 * Drop-in replacement for the per-node ionic update of KIT-IBT/CardioMechanics: the loop
 *     for each local node l:  dVm[l] = pem[l]->Calc(dtcell, Vm[l], i_ext[l], stretch[l], 1)
 * in acCELLerate::CalcCellModels (electrophysiology/src/acCELLerate/acCELLerate.cpp:1757-1770)
 * and the single-cell driver's `Vm += Calc(...)` (electrophysiology/src/CellModel/CellModel.h:420)
 * becomes one cm_batch_step() (or a fused multi-step cm_batch_run()) over all nodes on one GPU.
 *
 * Models: ten Tusscher-Panfilov 2006 ("TenTusscher2") and Courtemanche 1998 ("CourtemancheEtAl").
 * Units are the reference's: Vm and dVm in volts, dt in seconds, i_ext in nA per cell for
 * TenTusscher2 (TenTusscher2.cpp:630) and pA/pF for CourtemancheEtAl (CourtemancheEtAl.h:52).
 *
 * Conventions
 *  - Every call returns CM_OK (0) or a negative cm_status; cm_last_error() describes the last
 *    failure of the calling thread. No C++ exception crosses this boundary.
 *  - Array arguments are plain pointers to n_cells elements. They may be host memory
 *    (pageable or pinned) or device memory; the library tells them apart with
 *    cudaPointerGetAttributes and copies host arrays in and out on the batch's stream.
 *    Host arrays are only borrowed for the duration of the call.
 *  - `stream` arguments are cudaStream_t values (NULL = the legacy default stream). Calls
 *    that return host data synchronise that stream before returning.
 *  - A batch is not thread-safe; different batches are independent.
 */
#ifndef CARDIOMECH_GB300_H
#define CARDIOMECH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CM_ABI_VERSION 1

/* Model identifiers: the reference's ElphyModelType values (CellModel/ElphyModelBasis.h:62-81). */
typedef enum {
  CM_MODEL_COURTEMANCHE = 2, /* EMT_CourtemancheEtAl */
  CM_MODEL_TENTUSSCHER2 = 5  /* EMT_TenTusscher2 */
} cm_model;

typedef enum {
  CM_OK = 0,
  CM_ERR_ARG = -1,         /* bad argument (null handle, size, dt mismatch ...) */
  CM_ERR_MODEL = -2,       /* model not implemented here */
  CM_ERR_FILE = -3,        /* .ev file missing or malformed (CellModelValues.h:153-243) */
  CM_ERR_PARAM = -4,       /* unknown or missing parameter name */
  CM_ERR_CUDA = -5,        /* CUDA runtime failure (message in cm_last_error) */
  CM_ERR_NOMEM = -6,       /* device or host allocation failed */
  CM_ERR_UNSUPPORTED = -7, /* valid request this build does not serve */
  CM_ERR_NUMERIC = -8      /* NaN / out-of-range Vm detected by a fused check */
} cm_status;

/* Arithmetic form of a batch. */
typedef enum {
  CM_PREC_FP64 = 0,  /* every operation in FP64, the reference's arithmetic */
  CM_PREC_MIXED = 1  /* FP32 gates and currents; Vm, [Na]i, [K]i, [Ca]SR (Courtemanche: [Ca]up,
                        [Ca]rel) accumulated as compensated FP32 pairs (hi + lo); buffered-Ca
                        quadratics solved in a cancellation-free increment form */
} cm_precision;

/* State layouts for cm_batch_get_state / cm_batch_set_state. */
typedef enum {
  /* The reference backup block of every cell, cell after cell, byte-compatible with
   * vbElphyModel::GetBase()/GetSize() (TenTusscher2: 36 doubles = 288 B; Courtemanche:
   * 22 doubles = 176 B). Diagnostic slots (TT2 Array[18], CRN I_SAC) are written as
   * the library last computed them when diagnostics are on, else 0. */
  CM_LAYOUT_REF_BLOCK = 0,
  /* Structure of arrays: n_state_vars arrays of n_cells doubles, in cm_model_info order. */
  CM_LAYOUT_SOA = 1
} cm_layout;

/* Per-cell audit bits, OR-ed into the batch's audit mask by the kernels. */
enum {
  CM_AUDIT_NAN = 1u,          /* non-finite Vm or state after the step */
  CM_AUDIT_VRANGE = 2u,       /* voltage index outside the lookup table: clamped */
  CM_AUDIT_CARANGE = 4u,      /* [Ca]i index outside the ECa table (TT2): clamped */
  CM_AUDIT_GATE = 8u,         /* a gate left [0, 1] */
  CM_AUDIT_SURROGATE = 16u,   /* surrogate step rejected; plain integrator used */
  CM_AUDIT_VMRANGE = 32u,     /* |Vm| above the caller's vm_range after a fused update */
  CM_AUDIT_TIMEOUT = 64u,     /* a bounded device wait (bulk copy, tensor-core completion) ran
                                 out: the kernel left its remaining work undone and returned */
  CM_AUDIT_STAGE = 128u,      /* batched launch: a staged descriptor was not its tile's
                                 instance's; that sub-tile was skipped */
  CM_AUDIT_TILE = 256u        /* batched launch: a sub-tile outside its instance; skipped */
};

typedef struct cm_params_s *cm_params_t;
typedef struct cm_batch_s *cm_batch_t;

typedef struct {
  int model;           /* cm_model */
  int n_state_vars;    /* state variables in the SOA layout (Vm excluded) */
  int ref_block_doubles; /* GetSize()/8 of the reference model */
  int n_tables;        /* voltage-indexed lookup tables */
  int table_rows;      /* 4000 (RangeTab * DivisionTab, ElphyModelBasis.h:50-54) */
  double dt;           /* time step the tables were built for [s] */
  double init_vm;      /* GetVm() [V] */
  double amplitude;    /* GetAmplitude(): default stimulus amplitude */
  double stim_time;    /* GetStimTime(): default stimulus duration [s] */
} cm_info;

/* Stimulus protocol evaluated on the device by cm_batch_run, per cell as the reference
 * driver does (CellModel.h:405-419): i_ext = amplitude while t >= textbegin; at the first
 * step with t >= textbegin + textlen the stimulus is still applied and textbegin advances
 * by bcl. t starts at t0 and accumulates t += dt in FP64. */
typedef struct {
  double t0;
  double textbegin;           /* first stimulus time [s] (all cells) */
  /* Optional per-cell first stimulus time, overrides textbegin. A device array is the driver's
   * per-cell textbegin state: the run advances it in place, so the next call continues from it.
   * A host array is only read (the run advances a copy). */
  const double *textbegin_per_cell;
  double textlen;             /* stimulus duration [s] */
  double bcl;                 /* basic cycle length [s] */
  double amplitude;           /* reference units of i_external */
} cm_stimulus;

/* ------------------------------------------------------------------ library */
int cm_abi_version(void);
const char *cm_last_error(void);
/* Model type by reference name (FindElphyModelType, ElphyModelBasis.h:112-118); -1 if unknown. */
int cm_model_from_name(const char *name);
/* cm_info without a parameter set: n_state_vars, ref_block_doubles, n_tables, table_rows. */
int cm_model_info(int model, cm_info *info);
/* Name of SOA state variable k (k < n_state_vars). NULL if out of range. */
const char *cm_state_name(int model, int k);

/* ------------------------------------------------------------------ parameter sets */
/* initElphyParameters (CellModel/CellModelLayer.h:88-150): load an .ev parameter file and
 * build the lookup tables for time step dt [s] (TenTusscher2Parameters.cpp:384-524,
 * CourtemancheParameters.cpp:282-395). ev_path NULL selects the built-in defaults
 * (TenTusscher2_original_Epi.ev / CourtemancheEtAl.ev values). A parameter the model
 * needs but the file lacks is an error (the reference warns and uses -1). */
int cm_params_create(cm_params_t *out, int model, const char *ev_path, double dt);
int cm_params_destroy(cm_params_t p);
int cm_params_info(cm_params_t p, cm_info *info);
/* Named parameter value (base or derived, as the reference's P[] array holds it). */
int cm_params_get(cm_params_t p, const char *name, double *value);
/* Change a base parameter; derived values and tables are rebuilt (Calculate + InitTable). */
int cm_params_set(cm_params_t p, const char *name, double value);
/* Copy lookup table `name` (table_rows doubles) as built on the host in FP64. */
int cm_params_table(cm_params_t p, const char *name, double *out);

/* ------------------------------------------------------------------ batches of cells */
/* initElphyModel x n_cells (CellModelLayer.h:154-232) + Init(): device-resident state for
 * n_cells cells of the parameter set's model, initialised from its init values. The batch
 * keeps its own copy of the parameter set and tables. stream: cudaStream_t or NULL. */
int cm_batch_create(cm_batch_t *out, cm_params_t p, int64_t n_cells, int precision, void *stream);
int cm_batch_destroy(cm_batch_t b);
int cm_batch_info(cm_batch_t b, cm_info *info, int64_t *n_cells, int *precision);
/* Back to the initial state (vbElphyModel::Init for every cell). */
int cm_batch_reset(cm_batch_t b);
/* AddHeteroValue(name, values[c]) for every cell c (ElphyModelBasis.h:319-322): absolute
 * per-cell values of a parameter read in Calc. Supported names:
 *   TenTusscher2:     g_Na g_Kr g_K1 g_Ks g_to g_CaL
 *   CourtemancheEtAl: g_Na g_to g_Ks g_CaL g_bNa g_bCa
 * Others return CM_ERR_UNSUPPORTED. values == NULL removes the override. */
int cm_batch_set_hetero(cm_batch_t b, const char *name, const double *values);
/* Keep the reference's diagnostic values (TenTusscher2 Array[0..16] currents, Courtemanche
 * I_SAC) on the device so that CM_LAYOUT_REF_BLOCK state reads carry them. FP64 batches only;
 * costs 17 (TT2) or 1 (CRN) extra FP64 writes per cell-step while on. */
int cm_batch_set_diagnostics(cm_batch_t b, int on);
/* GetVm() for every cell into Vm (n_cells doubles). */
int cm_batch_init_vm(cm_batch_t b, double *Vm);
/* State transfer in the given cm_layout; buf holds n_cells * (ref_block_doubles or
 * n_state_vars) doubles. */
int cm_batch_get_state(cm_batch_t b, int layout, double *buf);
int cm_batch_set_state(cm_batch_t b, int layout, const double *buf);

/* One cell of a batch, for per-node code written against vbElphyModel (the slow path; the
 * C++ view in cardiomech_gb300_elphy.hpp is built on these three). */
/* The cell's state as GetBase()/GetSize() hold it (CM_LAYOUT_REF_BLOCK: ref_block_doubles
 * doubles, diagnostic slots as in cm_batch_get_state) or its n_state_vars values (SOA order).
 * out: host memory. Replaces reading vbElphyModel::GetBase() (ElphyModelBasis.h:206-207). */
int cm_batch_get_cell(cm_batch_t b, int64_t cell, int layout, double *out);
/* Writes one cell's state from a block in the given layout (host memory): ReadStatus / Set
 * into that cell (ElphyModelBasis.h:243-253). Diagnostic slots of a block are not read. */
int cm_batch_set_cell(cm_batch_t b, int64_t cell, int layout, const double *in);
/* One Calc of one cell, *dV = Calc(dt, V, i_ext, stretch, 1) (ElphyModelBasis.h:264), its
 * state updated in place on the device: vbElphyModel::Calc for node `cell`. dt must equal the
 * parameter set's dt. One launch and two small copies per call: use cm_batch_step for loops. */
int cm_batch_calc_cell(cm_batch_t b, int64_t cell, double dt, double V, double i_ext, double stretch, double *dV);
/* Column names after "t" and "V_m" of vbElphyModel::Print (long_form 0) or LongPrint (1), as
 * GetParameterNames / GetLongParameterNames give them (TenTusscher2.cpp:959-999,
 * CourtemancheEtAl.cpp:241-265, OHaraRudy.cpp:693-740, Tomek.cpp:686-733). Returns the count;
 * names (NULL: count only) receive static strings. */
int cm_model_print_names(int model, int long_form, const char **names, int cap);
/* The same columns' values for one cell at membrane voltage V [V] (Print / LongPrint:
 * TenTusscher2.cpp:908-957, CourtemancheEtAl.cpp:189-239, OHaraRudy.cpp:665-691,
 * Tomek.cpp:658-684), as the reference prints them after t and V. Stored values (TT2
 * Array[0..16], Courtemanche I_SAC, the O'Hara-Rudy and Tomek currents and Tomek's I_Na rates)
 * are those of the last step of an FP64 batch with diagnostics on (cm_batch_set_diagnostics),
 * else 0. Returns the count. */
int cm_batch_print_values(cm_batch_t b, int64_t cell, double V, int long_form, double *values, int cap);

/* One Calc for every cell: dVm[c] = Calc(dt, Vm[c], i_ext[c], stretch[c], 1), state updated
 * in place (acCELLerate.cpp:1757-1770). dt must equal the parameter set's dt (the tables
 * bake it in; the reference would silently use stale tables). i_ext NULL = no stimulus;
 * stretch NULL = 1.0. dVm may alias neither Vm nor i_ext. */
int cm_batch_step(cm_batch_t b, double dt, const double *Vm, const double *i_ext, const double *stretch,
                  double *dVm);

/* cm_batch_step fused with the caller's Godunov update and check (acCELLerate.cpp:1930-1949):
 * Vm[c] += Calc(dt, Vm[c], i_ext[c], stretch[c], 1), Vm updated in place. Returns
 * CM_ERR_NUMERIC when a new Vm is NaN/inf or |Vm| > vm_range (vm_range <= 0: no range check);
 * the offending cells carry CM_AUDIT_NAN / CM_AUDIT_VMRANGE in cm_batch_audit. */
int cm_batch_step_update(cm_batch_t b, double dt, double *Vm, const double *i_ext, const double *stretch,
                         double vm_range);
/* cm_batch_step_update with acCELLerate::IntraStep's activation times fused into the same pass
 * (acCELLerate.cpp:1997-2005): a cell whose act_time entry is still -1 and whose new Vm reaches
 * act_threshold [V] gets act_time = t [s]. act_time: n_cells doubles, host or device, updated in
 * place. The reference checks the Vm after its diffusion solve; this checks the Vm after the
 * reaction step, which is the same Vm when the step is the whole update (single cells, reaction-
 * only runs, or a splitting whose diffusion follows and is checked by the caller). */
int cm_batch_step_update_act(cm_batch_t b, double dt, double *Vm, const double *i_ext, const double *stretch,
                             double vm_range, double *act_time, double t, double act_threshold);

/* n_steps of the driver loop fused on the device: i_ext from the stimulus protocol,
 * Vm[c] += Calc(dt, Vm[c], i_ext, 1, 1) (CellModel.h:405-420). Vm is updated in place.
 * probe_cells (optional, n_probe indices) and probe_vm (n_probe * ceil(n_steps/probe_every))
 * record Vm before every probe_every-th step, probe-major. Returns CM_ERR_NUMERIC when a
 * cell's Vm became non-finite (the reference driver throws "Vm is NaN", CellModel.h:421). */
int cm_batch_run(cm_batch_t b, double *Vm, int64_t n_steps, const cm_stimulus *stim,
                 const int64_t *probe_cells, int64_t n_probe, int64_t probe_every, double *probe_vm);

/* Autotuner: times every launch shape of the batch's kernel (threads per block, register
 * budget, grid mode) on the batch itself for n_trial_steps steps each and keeps the fastest.
 * The batch's state and audit bits are saved before and restored after, so tuning does not
 * advance the cells. variant / ms_per_step (either may be NULL) receive the choice and its
 * time per step. FP64 batches have a single shape. */
int cm_batch_autotune(cm_batch_t b, int n_trial_steps, int *variant, double *ms_per_step);
/* Fix the launch shape: variant in [0, n) from cm_batch_autotune's set, grid_mode 0 (one
 * thread per cell) or k > 0 (grid-stride loop over k blocks per SM). */
int cm_batch_set_launch(cm_batch_t b, int variant, int grid_mode);

/* OR of the per-cell audit bits since the last call; per_cell (optional, n_cells uint32)
 * receives each cell's bits. Clears the bits. */
int cm_batch_audit(cm_batch_t b, uint32_t *mask, uint32_t *per_cell);

/* ------------------------------------------------------------------ monodomain coupling */
/* The explicit monodomain step of acCELLerate::IntraStep (acCELLerate.cpp:1839-2005, the
 * path without a mass matrix, Gauss points or implicit smoothing, Godunov current scheme):
 *     B = Intra.A * Vm                                   (MatMult, line 1849)
 *     i_ext[l] = scale[l] * B[l] + stimulus[l]           (nA/cell conversion 1880-1887,
 *                                                         injected-current conditions 1892)
 *     dVm[l] = Calc(dtcell, Vm[l], i_ext[l], 1, 1)       (CalcCellModels 1757-1770)
 *     Vm[l] += dVm[l], NaN / vm_def_range check          (1930-1949)
 *     activation times                                   (1997-2005)
 * with the matrix-vector product, the cell update, the check and the activation times fused
 * into one pass over the nodes per step. The reference's scale is -Volume()/volume_local*1e9. */
typedef struct cm_diffusion_s *cm_diffusion_t;

/* A: n x n in CSR (rowptr[n + 1] with rowptr[0] = 0, col[rowptr[n]] in [0, n), val), host
 * memory, as MatGetRowIJ / MatSeqAIJGetArray give it; the library keeps its own device copy
 * (slices of 32 rows stored column-major within the slice, so consecutive nodes' entries are
 * adjacent). scale: n doubles (host), or NULL for uniform_scale at every node. Row l of A
 * belongs to cell l of the batches it is used with. CM_ERR_ARG for malformed CSR. */
int cm_diffusion_create(cm_diffusion_t *out, int64_t n, const int64_t *rowptr, const int32_t *col,
                        const double *val, const double *scale, double uniform_scale);
int cm_diffusion_destroy(cm_diffusion_t d);
/* y[l] = scale[l] * (A x)[l] in FP64, entries summed in CSR order. x, y: n doubles, host or
 * device, not aliased. */
int cm_diffusion_apply(cm_diffusion_t d, const double *x, double *y);

/* n_steps monodomain steps (above) of batch b coupled by d (same n), fused on the device. Vm:
 * n doubles, host or device, updated in place; each step's product reads the previous step's
 * Vm of every node (the new values go to a second buffer). stim: the driver's stimulus protocol
 * as in cm_batch_run, whose current is added to i_ext (per-cell first-stimulus times give
 * regional stimuli: a cell with textbegin beyond the run is never stimulated). FP64 batches form
 * A*Vm in FP64 in CSR order; mixed batches in FP32 as rowsum(A)_l Vm_l + sum_j A_lj (Vm_j - Vm_l)
 * (no cancellation of the large diagonal). vm_range > 0: |Vm| beyond it is an error, as
 * vm_def_range. act (optional, n doubles, host or device): cells whose entry is -1 and whose new
 * Vm reaches act_threshold [V] get the step's time. Returns CM_ERR_NUMERIC if a Vm became
 * non-finite or left the range. */
int cm_batch_run_diffuse(cm_batch_t b, cm_diffusion_t d, double *Vm, int64_t n_steps, const cm_stimulus *stim,
                         double vm_range, double *act, double act_threshold);

/* ------------------------------------------------------------------ implicit step */
/* The finite-element path of acCELLerate::IntraStep (IntraRHS set, acCELLerate.cpp:1951-1993):
 * after the cell update, b = R x and the solve A x = b with A = C_m beta/dt M + theta K (the
 * reference's Intra.A) and R = C_m beta/dt M - (1 - theta) K (its IntraRHS), both given as
 * cm_diffusion_t operators built with uniform_scale 1 (the handle borrows them: destroy it
 * first). A must be symmetric positive definite with a positive diagonal: the solve is
 * conjugate gradients with the Jacobi preconditioner in FP64 from the current x as initial guess
 * (the reference: GMRES with block Jacobi, nonzero initial guess, PETScLSE.h:370-381), stopped
 * by PETSc's default test on the preconditioned residual, ||D^-1 r|| < max(rtol ||D^-1 b||,
 * atol), after max_iter iterations, or as divergence at dtol = 1e4 (acCELLerate.cpp:19-24 use
 * rtol = atol = 1e-6, max_iter = 1000). */
typedef struct cm_theta_s *cm_theta_t;
typedef struct {
  int64_t solves;          /* solves accounted */
  int64_t iterations;      /* their iterations in total */
  int64_t max_iterations;  /* the most any of them took */
  int64_t not_converged;   /* solves that ended without meeting the test */
  double last_norm;        /* the last solve's final preconditioned residual norm */
} cm_theta_stats;

int cm_theta_create(cm_theta_t *out, cm_diffusion_t lhs, cm_diffusion_t rhs, double rtol, double atol,
                    int max_iter);
int cm_theta_destroy(cm_theta_t t);
/* x <- A^-1 (R x); x: n doubles, host or device. stats (may be NULL) accumulates. CM_ERR_NUMERIC
 * when the solve diverged or broke down; a solve that ran out of iterations returns CM_OK and
 * counts in stats->not_converged (the reference prints a warning and goes on). */
int cm_theta_solve(cm_theta_t t, double *x, cm_theta_stats *stats);
/* n_steps implicit monodomain steps of batch b: the cell update with the stimulus protocol (as
 * cm_batch_run; no coupling current on this path), Vm += dVm with the range check (vm_range > 0),
 * the solve, and activation times after it (act: n doubles or NULL; entries -1 whose new Vm
 * reaches act_threshold get the step's time). Vm: n doubles, host or device, updated in place. */
int cm_batch_run_theta(cm_batch_t b, cm_theta_t t, double *Vm, int64_t n_steps, const cm_stimulus *stim,
                       double vm_range, double *act, double act_threshold, cm_theta_stats *stats);

/* ------------------------------------------------------------------ backup files */
/* acCELLerate backup files (acCELLerate::WriteBackup / ReadBackup, acCELLerate.cpp:1511-1661):
 * the line "acCELLerateBackupVersion1.0", the line "<time> <number of nodes>", then for every
 * node in order its Vm (one double) and its cell model's block (GetBase()/GetSize(): the
 * CM_LAYOUT_REF_BLOCK doubles), in the machine's byte order as the reference writes them on
 * Linux x86-64 and aarch64 (kaWrite swaps bytes only where KA_LITTLE_ENDIAN is defined,
 * Lattice/kaMachineOS.h:91-92, i.e. 32-bit x86). One file covers all parts (the materials'
 * batches): part p holds the nodes node_ids[p][0 .. n_cells-1] (global indices), or, when
 * node_ids or node_ids[p] is NULL, the next n_cells nodes after the previous part's. Every node
 * 0 .. n_total-1 must belong to exactly one part. Vm[p]: that part's n_cells values (host or
 * device). A block's stored currents are what cm_batch_get_state gives (zero unless the FP64
 * batch keeps diagnostics); reading takes the states and ignores them, as Calc overwrites them. */
int cm_backup_write(const char *path, const char *time_str, int n_parts, const cm_batch_t *parts,
                    const int64_t *const *node_ids, const double *const *Vm);
/* Reads such a file into the parts (their states and Vm). Checks the version line (as the
 * reference, case-insensitively), the node count against the parts' total and the file size
 * against the parts' block sizes (acCELLerate.cpp:1575-1578): CM_ERR_FILE on any mismatch.
 * time_out (may be NULL) receives the time string, at most time_cap bytes with the NUL. */
int cm_backup_read(const char *path, int n_parts, const cm_batch_t *parts, const int64_t *const *node_ids,
                   double *const *Vm, char *time_out, size_t time_cap);

/* ------------------------------------------------------------------ batched form */
/* Many batches (instances) of uneven size and mixed model -- e.g. the per-material cell
 * populations of acCELLerate (acltCellModel.cpp:64-126) or independent simulations -- advanced
 * together: one persistent kernel launch per time step over tiles of all instances, each
 * instance with its own stimulus protocol kept on the device, consecutive steps replayed from
 * a CUDA graph. The instances stay owned by the caller and keep working on their own. Only
 * CM_PREC_MIXED batches; each instance below 8e7 cells. */
typedef struct cm_multi_s *cm_multi_t;

int cm_multi_create(cm_multi_t *out, const cm_batch_t *batches, int n_batches, void *stream);
int cm_multi_destroy(cm_multi_t m);
/* n_steps of every instance's driver loop (CellModel.h:405-420) in lock step. Vm[i] points at
 * instance i's n_cells Vm values (host or device), updated in place; stims[i] is its protocol
 * (textbegin_per_cell not supported here). Returns CM_ERR_NUMERIC when a Vm became NaN. */
int cm_multi_run(cm_multi_t m, double *const *Vm, int64_t n_steps, const cm_stimulus *stims);
/* Autotuner of the batched launch: tries tile sizes, block shapes and grid sizes on the
 * instances themselves (states saved and restored) and keeps the fastest. Any output may be
 * NULL. */
int cm_multi_autotune(cm_multi_t m, int n_trial_steps, int *tile_cells, int *shape, int *blocks_per_sm,
                      double *ms_per_step);
int cm_multi_set_launch(cm_multi_t m, int tile_cells, int shape, int blocks_per_sm);

/* ------------------------------------------------------------------ learned macro step */
/* New with this library; the reference has no learned component. A ten Tusscher 2006
 * macro step of S fine steps = one physics step with tables for S * dt + an MLP correction
 * (22 -> 128 -> 128 -> 19, tanh, BF16 tensor-core GEMMs with FP32 accumulation, FP32 Adam)
 * trained on the residual of S fine steps of the plain integrator. The plain integrator
 * takes stimulated cells, the upstroke (|dVm/dt| > 5 mV/ms), cells failing the range audit
 * and a rotating audit sample, and measures the surrogate against itself on that sample. */
typedef struct cm_mlp_s *cm_mlp_t;
/* Parameter order of get/set: W1[n_hidden][n_in] b1[n_hidden] W2[n_hidden][n_hidden]
 * b2[n_hidden] W3[n_out][n_hidden] b3[n_out], FP32. Arrays may be host or device memory. */
int cm_mlp_create(cm_mlp_t *out, int n_in, int n_hidden, int n_out, uint64_t seed, void *stream);
int cm_mlp_destroy(cm_mlp_t m);
int64_t cm_mlp_n_params(cm_mlp_t m);
int cm_mlp_get_params(cm_mlp_t m, float *params);
int cm_mlp_set_params(cm_mlp_t m, const float *params);
/* Gradients of the last cm_mlp_loss_grad, same order as the parameters. */
int cm_mlp_get_grads(cm_mlp_t m, float *grads);
/* Y[n][n_out] = MLP(X[n][n_in]). */
int cm_mlp_forward(cm_mlp_t m, const float *X, int64_t n, float *Y);
/* Same result as cm_mlp_forward, for callers that must not allocate device memory during the
   call: a host code whose pool allocator owns the whole device, or a time-stepping loop that
   must not meet the device-wide synchronisation of cudaMalloc/cudaFree. No counterpart in the
   reference (its cell models have no network). X (n x n_in) and Y (n x n_out) must be device
   arrays; host arrays are rejected with CM_ERR_ARG, because staging them would allocate. The
   intermediates live in one fixed 8 MiB __device__ array per device, so n is limited to
   8 MiB / (2*(in_pad + 2*n_hidden) + 4*out_pad) bytes per row, rounded down to a multiple of 64
   (11,904 rows for the 22-128-128-19 surrogate network, in_pad = out_pad = 32); larger n is
   rejected with CM_ERR_ARG and a message giving the limit. Nothing in that array has to start
   at zero. The first call on a device (with that device current) looks the array's address up
   and loads it there; make that first call before any stream capture. The looked-up address is
   kept for the life of the process: it assumes the device's primary context lives as long as
   the process (no cudaDeviceReset between calls). The current device must be the one the
   network was created on; otherwise the call returns CM_ERR_ARG. The array is shared by
   every caller in the process: two calls that overlap in time, from two threads or on
   unordered streams, corrupt each other's results. Runs on the MLP's stream and returns after
   it has finished, like cm_mlp_forward. */
int cm_mlp_forward_static(cm_mlp_t m, const float *X, int64_t n, float *Y);
/* Mean squared error over the n x n_out outputs against T and its gradients. */
int cm_mlp_loss_grad(cm_mlp_t m, const float *X, const float *T, int64_t n, float *loss);
int cm_mlp_adam_step(cm_mlp_t m, float lr, float beta1, float beta2, float eps);

typedef struct cm_surrogate_s *cm_surrogate_t;
typedef struct {
  int64_t cell_macro_steps; /* cells x macro steps run */
  int64_t surrogate;        /* advanced by the learned macro step */
  int64_t fallback;         /* advanced by the plain integrator (stimulus, upstroke, audit) */
  int64_t audited;          /* audit sample: surrogate prediction compared with the plain result */
  double max_audit_err_mv;  /* largest |Vm surrogate - Vm plain| over the audit sample [mV] */
  double ms_step_kernel;    /* device time of the macro-step kernel, summed over the call (CUDA events) */
  double ms_plain_kernel;   /* device time of the plain-integrator kernel for the listed cells, summed */
} cm_surrogate_stats;

/* TenTusscher2 parameter set p (its dt is the fine step); substeps fine steps per macro step. */
int cm_surrogate_create(cm_surrogate_t *out, cm_params_t p, int substeps, uint64_t seed, void *stream);
int cm_surrogate_destroy(cm_surrogate_t s);
/* The surrogate's network (borrowed handle, valid while s lives). */
int cm_surrogate_mlp(cm_surrogate_t s, cm_mlp_t *mlp);
/* Training data from the plain integrator: advances the MIXED TenTusscher2 batch b by n_macro
 * macro steps of its driver loop (Vm updated in place) and records, for every cell_stride-th
 * cell and every macro step outside the stimulus and the upstroke, the features and the
 * residual target; appends up to max_pairs pairs in total. n_pairs: pairs held afterwards. */
int cm_surrogate_generate(cm_surrogate_t s, cm_batch_t b, double *Vm, int64_t n_macro, const cm_stimulus *stim,
                          int64_t cell_stride, int64_t max_pairs, int64_t *n_pairs);
/* Fresh network weights drawn from seed (Glorot-uniform, zero biases) and the optimiser state
 * cleared; the training pairs are kept. Lets one dataset train several candidate networks
 * (seeds) so that a caller keeps the one with the smallest error on held-out cells. */
int cm_surrogate_reset_network(cm_surrogate_t s, uint64_t seed);
/* Number of pairs held; X (n x 22) / T (n x 19) receive them when not NULL. */
int cm_surrogate_dataset(cm_surrogate_t s, int64_t *n_pairs, float *X, float *T);
/* Feature/target normalisation from the data, then `steps` Adam steps on minibatches. Then
 * every output's R^2 on a subsample of the data decides whether its correction is applied
 * (R^2 >= 0) or the coarse step's value is kept: a correction the network predicts worse than
 * the mean residual is noise that would accumulate over the macro steps. */
int cm_surrogate_fit(cm_surrogate_t s, int batch, int steps, float lr, uint64_t seed, float *final_loss);
/* Trained surrogate as one FP32 blob, for saving and loading: feature means (22), inverse
 * standard deviations (22), target scales (19), applied correction scales (19, 0 where the
 * correction is not applied; a caller may zero more of them), the outputs' R^2 on the training
 * data (19), then the network's parameters as cm_mlp_get_params orders them. */
int64_t cm_surrogate_blob_size(cm_surrogate_t s);
int cm_surrogate_get_blob(cm_surrogate_t s, float *blob);
int cm_surrogate_set_blob(cm_surrogate_t s, const float *blob);
/* Mode bits of cm_batch_run_surrogate. */
enum {
  CM_SUR_COARSE_ONLY = 1, /* coarse step alone: the method without the network */
  CM_SUR_AUDIT_FP64 = 2   /* the audit repeats its S fine steps in FP64 (else in the mixed form) */
};
/* n_macro macro steps of the driver loop with the surrogate (MIXED TenTusscher2 batch; Vm in
 * place). mode 0: coarse step + network; CM_SUR_* bits change that. Cells with stimulus,
 * |dVm/dt| above 5 mV/ms or a step the range audit rejects take S plain fine steps instead.
 * Audit (audit_mod > 0): every audit_mod-th cell, rotating, whose learned step was accepted is
 * integrated again from the same initial state by the plain method (FP64 with
 * CM_SUR_AUDIT_FP64, else the mixed form), during the next macro step, and the learned Vm is
 * compared with the result (stats: audited, max_audit_err_mv). The audited cell keeps its
 * learned step. The last macro step's sample is audited by the next call (see
 * cm_surrogate_flush_audit), so a call's stats count the audits completed during it. */
int cm_batch_run_surrogate(cm_batch_t b, cm_surrogate_t s, double *Vm, int64_t n_macro, const cm_stimulus *stim,
                           int mode, int audit_mod, cm_surrogate_stats *stats);
/* The audit sample of a run's last macro step is audited by the next run's first macro step
 * (inside the same launch); this audits it now instead -- after the last run of a simulation --
 * and reports it in stats (audited, max_audit_err_mv; the other fields 0). mode: the
 * CM_SUR_AUDIT_FP64 bit chooses the audit's arithmetic. */
int cm_surrogate_flush_audit(cm_surrogate_t s, int mode, cm_surrogate_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* CARDIOMECH_GB300_H */
