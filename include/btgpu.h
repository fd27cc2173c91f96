/*
 * btgpu.h -- C ABI of the GB300 Bloch-Torrey finite-element engine (libbtgpu.so).
 *
 * The library replaces the arithmetic under the reference's solver call
 * (van-dang/DMRI-FEM-Cloud, DmriFemLib.py `MRI_simulation.solve`, lines
 * 878-915): the per-step DOLFIN `assemble(F)`/`assemble(L)` of the theta-method
 * forms (DmriFemLib.py:58-145, 904-905), the PETSc Krylov solve
 * (DmriFemLib.py:907; GCloudDmriSolver.py:219-222) and the signal functional of
 * `PostProcessing` (DmriFemLib.py:917-931).
 *
 * Conventions
 *  - Every function returns an int status: BT_OK (0) or one of BT_ERR_*.
 *    Nothing calls exit(); the text of the last failure is available from
 *    bt_last_error().
 *  - Host arrays are caller-owned and copied during the call.  Device memory,
 *    the stream, events and CUDA graphs belong to the context.
 *  - A context is not thread-safe: use one context per host thread.
 *  - Units follow the reference: lengths in um, times in us, D in um^2/us
 *    (numerically mm^2/s), kappa in um/us (numerically m/s), q = sqrt(b/int4gb).
 */
#ifndef BTGPU_H
#define BTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BT_OK 0
#define BT_ERR_INVALID 1        /* bad argument or mesh                      */
#define BT_ERR_CUDA 2           /* CUDA runtime error                        */
#define BT_ERR_OOM 3            /* device allocation failed                  */
#define BT_ERR_NOT_CONVERGED 4  /* a step hit max_iterations                 */
#define BT_ERR_BREAKDOWN 5      /* COCG breakdown (p^T A p = 0)              */
#define BT_ERR_TIMEOUT 6        /* a device-side wait ran out of time        */
#define BT_ERR_STATE 7          /* call out of order (e.g. solve before assemble) */

#define BT_PRECISION_FP64 0     /* FP64 matrices and Krylov vectors          */
#define BT_PRECISION_MIXED 1    /* FP32 inner COCG, FP64 residual/refinement/signal */

/* Matrices that bt_get_matrix() can export (values in CSR order). */
#define BT_MAT_M 0   /* int phi_i phi_j over the dof's compartment            */
#define BT_MAT_K 1   /* int D grad phi_i . grad phi_j                           */
#define BT_MAT_T 2   /* int (1/T2) phi_i phi_j                                  */
#define BT_MAT_R 3   /* kappa int_Gamma [phi_i][phi_j] on compartment interfaces */
#define BT_MAT_JX 4  /* int x phi_i phi_j                                       */
#define BT_MAT_JY 5  /* int y phi_i phi_j                                       */
#define BT_MAT_JZ 6  /* int z phi_i phi_j                                       */

typedef struct bt_ctx bt_ctx;

typedef struct bt_mesh_info_t {
    int64_t n_vertices;
    int64_t n_cells;
    int64_t n_dofs;              /* live (vertex, compartment) pairs            */
    int64_t nnz;                 /* CSR entries of the duplicated-node graph    */
    int64_t n_interface_facets;  /* facets between cells of different compartments */
    int32_t n_compartments;
    int32_t n_colours;           /* cell colours of the assembly               */
    int64_t sell_entries;        /* sliced-ELL slots (incl. padding)            */
    double volume;               /* sum of cell volumes                         */
} bt_mesh_info_t;

typedef struct bt_periodic_info_t {
    int32_t active;              /* 1 when a periodic direction is set          */
    int32_t dir[3];              /* PeriodicDir                                 */
    double kappa_e;              /* penalty 3e-3 / hmin                         */
    double hmin;                 /* smallest cell diameter                      */
    int64_t n_facets;            /* exterior facets with a nonzero penalty      */
    int64_t n_rows;              /* dofs with a mirror term                     */
    int64_t n_entries;           /* mirror-term entries                         */
    int64_t n_unmatched;         /* mirror points outside every face triangle   */
} bt_periodic_info_t;

typedef struct bt_stats_t {
    int32_t steps;               /* time steps per signal                       */
    int32_t max_iterations;      /* largest inner iteration count of any step   */
    int64_t total_iterations;    /* inner iterations summed over steps/signals  */
    double max_rel_residual;     /* largest final ||r||/||b|| over steps        */
    double gpu_ms;               /* device time of the solve (CUDA events)      */
    int32_t refinements;         /* mixed precision: outer sweeps, summed       */
    int32_t graph_launches;      /* solves replayed from a captured CUDA graph  */
    int64_t kernel_launches;     /* kernels launched by the solve               */
    double stepper_ms;           /* device time of the time-stepping kernels    */
} bt_stats;

/* Library version (major*10000 + minor*100 + patch). */
int bt_version(void);

/* Create a context on CUDA device `device`.  Replaces nothing in the
 * reference: DOLFIN objects are created implicitly by the Python API
 * (DmriFemLib.py:583-637). */
int bt_create(bt_ctx** out, int device);
int bt_destroy(bt_ctx* ctx);

/* Copy the last error text (NUL-terminated, truncated to len). */
int bt_last_error(const bt_ctx* ctx, char* buf, size_t len);

/* Run the context's work on a caller-provided cudaStream_t (NULL restores the
 * context's own stream). */
int bt_set_stream(bt_ctx* ctx, void* cuda_stream);

/* Upload a tetrahedral P1 mesh and build the duplicated-interface-node graph on
 * the device (CSR + sliced-ELL, cell colouring).  Replaces DOLFIN's mesh read
 * and function spaces: GCloudDmriSolver.py:150-152, MyFunctionSpaces
 * (DmriFemLib.py:453-486), phase = marker % 2 (DmriFemLib.py:764).
 *   xyz[n_vertices*3], tets[n_cells*4] (0-based), cell_region[n_cells] in
 *   [0,n_regions), region_compartment[n_regions] (NULL: region % 2, the
 *   reference's phase). */
int bt_mesh_upload(bt_ctx* ctx, const double* xyz, int64_t n_vertices,
                   const int32_t* tets, int64_t n_cells,
                   const int32_t* cell_region, int32_t n_regions,
                   const int32_t* region_compartment);

int bt_mesh_info(bt_ctx* ctx, bt_mesh_info_t* out);

/* Per-region coefficients.  D_region[n_regions] isotropic D
 * (mydomain.D, DmriFemLib.py:611-616; GCloudDmriSolver.py:207-215);
 * invT2_region[n_regions] 1/T2 (NULL: 0, the reference default T2=1e16,
 * DmriFemLib.py:807); kappa_pair[n_regions*n_regions] permeability between
 * two regions (NULL: 0; mydomain.kappa, GCloudDmriSolver.py:204, or the
 * per-interface values of MultilayeredDiskVariablePermeability.ipynb:480-502). */
int bt_set_coefficients(bt_ctx* ctx, const double* D_region, const double* invT2_region,
                        const double* kappa_pair);

/* How the permeability enters the interface term kappa int_F [u][v] (icondition_wBC,
 * DmriFemLib.py:47-50): BT_KAPPA_FACET (default) uses the region pair's value,
 * constant on each interface facet (GCloudDmriSolver.py:204); BT_KAPPA_CR is the
 * reference's per-interface permeability as a Crouzeix-Raviart function
 * (MultilayeredDiskVariablePermeability.ipynb:480-502): the CR dof of every
 * interior facet is kappa_pair of its two regions where they differ, else 0, so
 * on a facet whose cell has another interface facet (staircase corners) kappa is
 * linear, not constant; the facet integral is then exact cubic.  Takes effect at
 * the next bt_assemble; bt_mesh_upload resets it.  The adjoints and bt_tangent
 * reject the CR mode. */
#define BT_KAPPA_FACET 0
#define BT_KAPPA_CR 1
int bt_set_kappa_mode(bt_ctx* ctx, int32_t mode);

/* Optional anisotropic per-cell D: D_cell[n_cells*6] = (xx, yy, zz, xy, xz, yz)
 * (ImposeDiffusionTensor, DmriFemLib.py:611-616, symmetric part).  NULL
 * clears it (back to D_region). */
int bt_set_cell_diffusion(bt_ctx* ctx, const double* D_cell);

/* Optional per-cell relaxation: invT2_cell[n_cells] = 1/T2 per cell (a DG0 T2
 * field, T2_Relaxation.ipynb; 0 = no decay), overriding invT2_region.  NULL
 * clears it.  bt_adjoint rejects per-cell T2 (its gradients are per region). */
int bt_set_cell_T2(bt_ctx* ctx, const double* invT2_cell);

/* Assemble M, K, T, R, Jx, Jy, Jz and the signal weights on the device with the
 * coloured, atomic-free element kernel.  Replaces the FFC tabulate_tensor +
 * PETSc insertion behind assemble() (DmriFemLib.py:245,252,904-905). */
int bt_assemble(bt_ctx* ctx);

/* Time schedule: f_new[n_sequences*n_steps] is f at the implicit level of
 * each solve, f_old[...] at the explicit level, exactly as the reference's
 * loop evaluates them (DmriFemLib.py:897-911: f(t) in F, f(tp) in L).
 * dt = mri_simu.k, theta = mri_simu.theta. */
int bt_set_schedule(bt_ctx* ctx, const double* f_new, const double* f_old,
                    int32_t n_steps, int32_t n_sequences, double dt, double theta);

/* Phase schedule of the pseudo-periodic boundary term: F_old[n_sequences*n_steps]
 * = F(tp) = int_0^tp f at the explicit level of each step (the itime_profile
 * value the reference passes to WeakPseudoPeriodic.set_values, DmriFemLib.py:
 * 73, 117, 901-905).  Sizes must equal the schedule's; bt_set_schedule clears
 * it.  Needed only when periodic directions are set. */
int bt_set_schedule_phase(bt_ctx* ctx, const double* F_old, int32_t n_steps, int32_t n_sequences);

/* Integral schedule of the strong pseudo-periodic form: F_new[n_sequences*n_steps]
 * = itime_profile(t) at the implicit level and F_old[...] = itime_profile(tp) at the
 * explicit level of each step (the ift arguments of ThetaMethodF/L_sBC1c/2c,
 * DmriFemLib.py:148-238, 897-905).  Also sets the weak form's phase schedule
 * (F_old).  Sizes must equal the schedule's; bt_set_schedule clears it. */
int bt_set_schedule_integral(bt_ctx* ctx, const double* F_new, const double* F_old, int32_t n_steps,
                             int32_t n_sequences);

/* Which pseudo-periodic form bt_set_periodic selects: BT_PERIODIC_WEAK (default,
 * IsDomainPeriodic = False) or BT_PERIODIC_STRONG (IsDomainPeriodic = True: the
 * constrained periodic space of MyFunctionSpaces with PeriodicBD,
 * DmriFemLib.py:325-378, 453-486, and the forms ThetaMethodF/L_sBC1c/2c,
 * DmriFemLib.py:148-238).  Applies to the directions already set and to later
 * bt_set_periodic calls; bt_mesh_upload resets it to weak.
 *
 * Strong form: the mesh must be periodic (every vertex of a max face has a
 * vertex at its image on the min face, within 1e-6 hmin) with periodic
 * compartments (a folded vertex touches the compartments of its image), at most
 * two compartments.  Pairing follows the reference's PeriodicBD: a max-face
 * vertex folds onto its image along the first periodic direction whose max face
 * holds it, nothing is chained (with several directions the edge columns
 * (xmax, ymin), (xmin, ymin) stay separate dofs, as in the reference).  Solved by
 * a persistent FP64 Jacobi-BiCGSTAB stepper (the operator has first-order terms
 * and is not complex symmetric) to ||r|| <= rtol ||b||; bt_solve needs
 * BT_PRECISION_FP64 and bt_set_schedule_integral.  A signal whose gradient has a
 * component along which (D g).n does not vanish on an exterior facet off the
 * periodic faces that touches a compartment interface is refused
 * (BT_ERR_INVALID): there the reference's phase-blind outer term acts on the
 * other compartment's dead rows, which one dof per live (vertex, compartment)
 * pair does not hold.  bt_get_solution returns the unfolded dofs (a folded dof's
 * value on each of its vertices).  The adjoints, bt_tangent and the mixed path
 * reject the strong form. */
#define BT_PERIODIC_WEAK 0
#define BT_PERIODIC_STRONG 1
int bt_set_periodic_mode(bt_ctx* ctx, int32_t mode);

/* Size of the folded system of the strong form after the last solve that set it
 * up: dofs, stored entries and vertex classes (0 when the strong form is off or
 * not set up yet). */
int bt_strong_periodic_info(bt_ctx* ctx, int64_t* n_dofs, int64_t* nnz, int64_t* n_classes);

/* Weak pseudo-periodic boundary conditions: periodic_dir[3] = mydomain.PeriodicDir
 * (0/1 per axis; all 0 or NULL switches them off), the reference's default
 * form when IsDomainPeriodic is False (ThetaMethodF/L_wBC1c/2c,
 * DmriFemLib.py:58-145, WeakPseudoPeriodic_1c/2c :256-323, :386-451,
 * WeakPseudoPeridicMarker :598-610).  The implicit matrix gains
 * theta int kappa_e u v ds, every step's right-hand side gains
 * (1-theta) int kappa_e ubc v ds with ubc = u_n at the mirror point on the
 * opposite face times exp(i q F(tp) g.shift).  The box is the mesh's bounding
 * box; the mesh need not be periodic.  Call after bt_mesh_upload (a new mesh
 * clears it).  With bt_set_periodic_mode(BT_PERIODIC_STRONG) the same call selects
 * the strong form instead (see there).  bt_adjoint and bt_tangent reject a
 * periodic context. */
int bt_set_periodic(bt_ctx* ctx, const int32_t* periodic_dir);
int bt_periodic_info(bt_ctx* ctx, bt_periodic_info_t* out);

/* Integrate n_signals Bloch-Torrey problems and return their signals.
 *   q[n_signals]            mri_para.qvalue
 *   gdir[n_signals*3]       unit gradient directions (set_gradient_dir)
 *   sequence[n_signals]     schedule row of each signal (NULL: all 0)
 *   u0[n_vertices]          initial condition (NULL: 1 everywhere, the
 *                           reference's Dirac_Delta, DmriFemLib.py:865-876)
 *   precision               BT_PRECISION_FP64 or BT_PRECISION_MIXED
 *   rtol, max_iterations    per-step COCG stopping rule ||r|| <= rtol ||b||
 *                           (linsolver relative_tolerance / maximum_iterations)
 *   signal_out[n_signals]   int Re(u(T)) dx   (PostProcessing `signal`)
 *   compartment_out         [n_signals*n_compartments] or NULL
 *   S0_out                  int u0 dx         (PostProcessing `voi`)
 * Replaces MRI_simulation.solve (DmriFemLib.py:878-915) and the signal of
 * PostProcessing (DmriFemLib.py:922-931). */
int bt_solve(bt_ctx* ctx, int32_t n_signals, const double* q, const double* gdir,
             const int32_t* sequence, const double* u0, int32_t precision,
             double rtol, int32_t max_iterations, double* signal_out,
             double* compartment_out, double* S0_out, bt_stats* stats);

/* bt_solve with device pointers (torch CUDA tensors, ...): d_q[n_signals],
 * d_gdir[n_signals*3], d_sequence[n_signals] (nullable), d_u0[n_vertices]
 * (nullable) are read from device memory and d_signal_out[n_signals],
 * d_compartment_out[n_signals*n_compartments] (nullable) written to it, on the
 * context's stream; S0_out and stats stay host pointers.  The per-signal
 * parameters and u0 are staged through the host (the solve validates them and
 * builds its schedule there); the caller keeps the arrays alive for the call,
 * which returns after the outputs are written.  Non-device pointers are
 * rejected (BT_ERR_INVALID). */
int bt_solve_dev(bt_ctx* ctx, int32_t n_signals, const double* d_q, const double* d_gdir,
                 const int32_t* d_sequence, const double* d_u0, int32_t precision, double rtol,
                 int32_t max_iterations, double* d_signal_out, double* d_compartment_out, double* S0_out,
                 bt_stats* stats);

/* Several meshes in one persistent launch (mixed precision): mesh m is the
 * mesh, coefficients, assembly and schedule of contexts[m] and gets
 * n_signals[m] (1..256) signals; q, gdir, sequence and signal_out list the
 * signals mesh by mesh.  The launch's blocks are split among the meshes in
 * proportion to their work; each mesh advances with its own grid barrier and
 * reductions, so meshes of uneven size and iteration count never wait for one
 * another.  u0 = 1 on every mesh; S0_out[n_meshes] (or NULL) receives the
 * volumes.  All contexts must be on one device; the work runs on the first
 * context's stream and errors are reported there.  At most 64 meshes.  The
 * reference integrates one mesh per MPI job (GCloudDmriSolver.py); it has no
 * batched counterpart. */
int bt_solve_multi(bt_ctx* const* contexts, int32_t n_meshes, const int32_t* n_signals,
                   const double* q, const double* gdir, const int32_t* sequence, double rtol,
                   int32_t max_iterations, double* signal_out, double* S0_out, bt_stats* stats);

/* Discrete adjoint of the FP64 solve of one signal: the signal and its
 * derivatives with respect to the per-region isotropic D (dS_dD[n_regions]),
 * 1/T2 (dS_dinvT2[n_regions]) and the permeability of each region pair
 * (dS_dkappa[n_regions*n_regions], symmetric: both entries of a pair hold the
 * derivative with respect to that pair's single value).  Derivatives are of
 * the unnormalised signal int Re(u(T)) dx; divide by S0 for the normalised
 * one.  Forward states are recomputed from checkpoints every
 * checkpoint_stride steps (0: ceil(sqrt(n_steps))).  The reference has no
 * adjoint; its gradients would be finite differences of MRI_simulation.solve
 * (DmriFemLib.py:878-915).  Any output pointer may be NULL. */
int bt_adjoint(bt_ctx* ctx, double q, const double* gdir, int32_t sequence, const double* u0,
               double rtol, int32_t max_iterations, int32_t checkpoint_stride,
               double* signal_out, double* dS_dD, double* dS_dinvT2, double* dS_dkappa,
               bt_stats* stats);

/* The same adjoint with per-cell fields: dS_dD_cell[n_cells*6] is the derivative
 * with respect to the stored components (xx, yy, zz, xy, xz, yz) of a per-cell
 * diffusion tensor (an off-diagonal component sets D_kl and D_lk together, as in
 * bt_set_cell_diffusion) and dS_dinvT2_cell[n_cells] with respect to a per-cell
 * 1/T2, both at the context's current coefficients (per-region or per-cell);
 * dS_dkappa as in bt_adjoint.  The derivative with respect to an isotropic D of
 * cell t is xx + yy + zz.  Any output pointer may be NULL. */
int bt_adjoint_cells(bt_ctx* ctx, double q, const double* gdir, int32_t sequence, const double* u0,
                     double rtol, int32_t max_iterations, int32_t checkpoint_stride,
                     double* signal_out, double* dS_dD_cell, double* dS_dinvT2_cell, double* dS_dkappa,
                     bt_stats* stats);

/* The same discrete adjoint for n_signals signals at once in the batched mixed
 * precision stepper (FP32 Krylov vectors, double-float residuals; the backward
 * sweep is a forward sweep of the same kernel with the schedule pair
 * f_new[n-1], f_old[n]): signal_out[n_signals], dS_dD[n_signals*n_regions],
 * dS_dinvT2[n_signals*n_regions], dS_dkappa[n_signals*n_regions*n_regions]
 * (signal-major, as bt_adjoint per signal).  u0 = 1.  Up to 256 signals share
 * one set of launches -- fewer when their checkpoint, segment and backward
 * states would take more than a quarter of the free device memory; more are
 * processed in groups.  Any output pointer but signal_out may be NULL. */
int bt_adjoint_batch(bt_ctx* ctx, int32_t n_signals, const double* q, const double* gdir,
                     const int32_t* sequence, double rtol, int32_t max_iterations, int32_t checkpoint_stride,
                     double* signal_out, double* dS_dD, double* dS_dinvT2, double* dS_dkappa, bt_stats* stats);

/* Per-cell gradients of a weighted sum of signals, sum_s weights[s] * S_s, by the
 * batched mixed-precision adjoint (bt_adjoint_batch's pipeline): dS_dD_cell[n_cells*6]
 * with respect to the stored components (xx, yy, zz, xy, xz, yz) of a per-cell
 * diffusion tensor, dS_dinvT2_cell[n_cells] with respect to a per-cell 1/T2 (both at
 * the context's current coefficients, per-region or per-cell) and
 * dS_dkappa[n_regions*n_regions] with respect to the pair permeabilities; the
 * signals themselves go to signal_out[n_signals].  This is the vector-Jacobian
 * product autograd needs for a field: weights = the incoming gradient.  Output
 * pointers other than signal_out may be NULL. */
int bt_adjoint_batch_cells(bt_ctx* ctx, int32_t n_signals, const double* q, const double* gdir,
                           const int32_t* sequence, const double* weights, double rtol, int32_t max_iterations,
                           int32_t checkpoint_stride, double* signal_out, double* dS_dD_cell, double* dS_dinvT2_cell,
                           double* dS_dkappa, bt_stats* stats);

/* bt_adjoint_batch for several meshes in one call: mesh m is the mesh,
 * coefficients, assembly and schedule of contexts[m] (all with the same number
 * of steps and theta) and gets n_signals[m] (1..256) signals; q, gdir, sequence
 * and signal_out list the signals mesh by mesh, and the gradients are
 * concatenated mesh by mesh in bt_adjoint_batch's layout: dS_dD and dS_dinvT2
 * hold n_signals[m] * n_regions(m) values per mesh, dS_dkappa n_signals[m] *
 * n_regions(m)^2.  Meshes whose batch fills the GPU run alone; the others share
 * every launch of the adjoint (forward with checkpoints, the w step, segment
 * recomputes and backward segments), each with its own sub-grid.  All work runs
 * on the first context's stream; at most 64 meshes.  The reference has no
 * adjoint: its gradients would be finite differences of one GCloudDmriSolver.py
 * job per mesh (GCloudDmriSolver.py:232, DmriFemLib.py:878-915). */
int bt_adjoint_multi(bt_ctx* const* contexts, int32_t n_meshes, const int32_t* n_signals, const double* q,
                     const double* gdir, const int32_t* sequence, double rtol, int32_t max_iterations,
                     int32_t checkpoint_stride, double* signal_out, double* dS_dD, double* dS_dinvT2,
                     double* dS_dkappa, bt_stats* stats);

/* Tangent-linear FP64 run: the signal and its derivative with respect to one
 * coefficient, param = BT_PARAM_D (D of region i), BT_PARAM_INVT2 (1/T2 of
 * region i) or BT_PARAM_KAPPA (permeability of the region pair (i, j)), by the
 * forward-mode recursion A_n v_{n+1} = B_n v_n - (dS/dparam)(theta u_{n+1} +
 * (1-theta) u_n), v_0 = 0.  A check of bt_adjoint (the two agree to solver
 * precision); keeps all forward states on the device.  No counterpart in the
 * reference (its derivatives would be finite differences). */
#define BT_PARAM_D 0
#define BT_PARAM_INVT2 1
#define BT_PARAM_KAPPA 2
int bt_tangent(bt_ctx* ctx, double q, const double* gdir, int32_t sequence, const double* u0,
               int32_t param, int32_t i, int32_t j, double rtol, int32_t max_iterations,
               double* signal_out, double* dsignal_out, bt_stats* stats);

/* Tuning knobs (no counterpart in the reference).  Keys:
 *   "mixed.lanes_per_row"   1,2,4,...,32 (0: autotune, the default)
 *   "mixed.blocks_per_sm"   co-resident blocks of the batched kernel (0: autotune)
 *   "mixed.max_sweeps"      refinement sweeps per step (default 8)
 *   "mixed.eps_first"       inner FP32 tolerance of the first sweep (3e-6)
 *   "mixed.eps_next"        inner FP32 tolerance of later sweeps (1e-2)
 *   "mixed.blocked_rows"    rows of a block: 1 contiguous range, 0 interleaved, -1 tuned (default)
 *   "mixed.divergence"      an FP32 inner sweep of a signal ends when its residual norm grows this
 *                           many times above the smallest it reached in the sweep (default 1e4)
 *   "mixed.reduce"          grid sums: 0 the last block to arrive sums and publishes, 1 every block sums
 *                           all partials itself, -1 by size (default; same bits either way)
 *   "mixed.extrapolate"     order of the initial guess of each step, extrapolated in time from the
 *                           last states: 4 (default), 3, 2 (3u_n - 3u_{n-1} + u_{n-2}),
 *                           1 (2u_n - u_{n-1}) or 0 (u_n)
 *   "mixed.inner_reductions" grid-wide reductions per inner COCG iteration: 1 (the
 *                           single-reduction rearrangement) or 2 (default, the textbook form); the
 *                           adjoint's and the pseudo-periodic launches always use 2
 *   "mixed.sort_signals"    1 (default): bt_solve's mixed path orders the signals by (sequence, |q|)
 *                           before cutting them into launches of 256 and warps of 32, so signals of
 *                           similar convergence share them (outputs keep the call's order); 0: as given
 *   "strong.batch"          1 (default): in the strong pseudo-periodic form, signals of one sequence
 *                           share batched launches (up to 32, one lane each, any directions; groups of
 *                           one or two run alone); 0: one launch per signal
 *   "fp64.extrapolate"      order of the FP64 path's initial guess, extrapolated in time from the
 *                           last states: 4 (default), 3, 2, 1 (2 u_n - u_{n-1}) or 0 (u_n); the strong
 *                           pseudo-periodic stepper uses 2 u_n - u_{n-1} for any order >= 1
 *   "fp64.pair_signals"     2 (default) or 1: bt_solve's FP64 path steps two signals of one gradient
 *                           direction (identical gdir rows; each signal is paired with the next
 *                           unpaired one of its direction) in one launch (shared matrix loads and grid
 *                           barriers, each signal with its own COCG scalars and stopping test); 2
 *                           runs one block per SM (~200 registers), 1 two blocks per SM (128
 *                           registers, a few spilled); 0: one launch per signal.  Not used with
 *                           weak pseudo-periodic boundaries.
 *   "fp64.blocks_per_sm"    blocks per SM of the FP64 one-signal stepper: -1 (default) one block per
 *                           SM while the mesh needs at most 4 x SMs blocks of one thread per row,
 *                           else as many as fit; 0: as many as fit; k >= 1: at most k (a warp then
 *                           takes more than one 32-row slice)
 * Failure detection (every device-side wait of the persistent steppers is
 * bounded; a wait that runs out ends the launch and the call returns
 * BT_ERR_TIMEOUT, leaving the context usable):
 *   "wait.limit_ns"         time limit of every grid-wide wait (default 2e9 = 2 s; 1e4 .. 6e10)
 *   "test.stall_first_wait" 1: every later solve's first wait is on a word nothing writes, so it
 *                           runs out after wait.limit_ns (exercises the timeout path); 0 (default) off */
int bt_set_option(bt_ctx* ctx, const char* key, double value);

/* Signal functional S = sum_i weights[i] * Re(u[i]) of a device-resident state,
 * computed without allocating any memory.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc when they read a signal (code running
 * inside CUDA stream capture, a serving or acquisition thread whose allocator is
 * frozen after start-up).  d_weights[n] are the per-dof signal weights
 * (bt_get_dofs), d_u[2n] the state as (re, im) pairs (bt_get_solution layout),
 * d_signal one double; all are device pointers.  Work is enqueued on
 * cuda_stream (NULL: the legacy default stream) of the current device.
 * Scratch is a static 8 KB device array: n <= 2097152, larger n returns
 * BT_ERR_INVALID.  The first call on each device looks up that array's device
 * address, so make it before any stream capture begins (the address is looked
 * up again when the device's context changes, e.g. after cudaDeviceReset, so
 * after a reset make one call before capturing, too).  Calls share the
 * scratch: calls that overlap on the GPU race and must be serialised.
 * Returns a status code only (no context, so no bt_last_error text). */
int bt_signal_noalloc(const double* d_weights, const double* d_u, int64_t n, double* d_signal,
                      void* cuda_stream);

/* Introspection for tests (no counterpart in the reference). */
int bt_get_csr(bt_ctx* ctx, int32_t* row_ptr /* n_dofs+1 */, int32_t* col /* nnz */);
int bt_get_matrix(bt_ctx* ctx, int32_t which, double* values /* nnz */);
int bt_get_dofs(bt_ctx* ctx, int32_t* dof_vertex, int32_t* dof_compartment, double* weights);
int bt_get_colouring(bt_ctx* ctx, int32_t* cell_colour /* n_cells */);
/* Final state of signal `index` of the last bt_solve: u[2*n_dofs] (re, im). */
int bt_get_solution(bt_ctx* ctx, int32_t index, double* u);
/* Per-step inner iteration counts of the last solve: iters[n_signals*n_steps];
 * capacity is the number of int32 the buffer holds. */
int bt_get_iterations(bt_ctx* ctx, int32_t* iters, int64_t capacity);

#ifdef __cplusplus
}
#endif

#endif /* BTGPU_H */
