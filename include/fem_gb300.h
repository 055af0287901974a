/*
 * fem_gb300.h -- C ABI of libfemgb300.so, the GB300 (sm_103a) implementation of
 * SolverFEM's per-substep hot path: Stable Neo-Hookean Tet4/Hex8 forces and
 * approximate PSD tangent, deterministic 3x3-block BSR assembly of
 * A = M + h^2 K~ + h C_s, and block-Jacobi preconditioned CG with the fixed-node
 * projection PAP + I - P.
 *
 * Reference interfaces replaced (paths inside the reference project,
 * src/newton_solver_fem/_src/solvers/fem/):
 *   fem_create / fem_destroy     SolverFEM.__init__                  solver.py:212-415
 *   fem_step                     SolverFEM.step                      solver.py:942-1002
 *   fem_refresh_tangent          SolverFEM.refresh_tangent           solver.py:769-857
 *   fem_rebuild_element_blocks   SolverFEM.rebuild_element_blocks    solver.py:506-508, 591-687
 *   fem_refresh_preconditioner   SolverFEM.refresh_preconditioner    solver.py:502-504
 *   fem_set_tolerance            SolverFEM.linear_solver_tolerance   solver.py:241-243, 1203-1217
 *   fem_set_maxiter              SolverFEM.linear_solver_maxiter     solver.py:273
 *   fem_reset                    SolverFEM.reset                     solver.py:436-443
 *   fem_velocity_increment_ptr   SolverFEM.velocity_increment        solver.py:478-481
 *   fem_get_stats                SolverFEM.last_cg_iters             solver.py:279, 1333-1335
 *   fem_eval_forces              SolverFEM.eval_*_forces             solver.py:1357-1600
 *   fem_set_soft_contacts        Contacts.soft_contact_* into step   solver.py:1540-1566
 *   fem_set_surface_contacts     SolverFEM.set_soft_surface_contacts solver.py:510-540
 *   fem_update_surface_contacts  SoftBodySurfaceContacts.update      soft_surface_contacts.py:226-237
 *   fem_prepare_tet_updates      SolverFEM.prepare_tetrahedral_updates solver.py:693-719
 *   fem_update_tet_topology      refresh_topology(element_sources=)   solver.py:872-940, streaming.py:549-700
 *   fem_export_bsr               SolverFEM.A_bsr (Warp BsrMatrix)    solver.py:322-337
 *   fem_export_preconditioner    SolverFEM._pc_inv_diag              solver.py:1142-1201
 *   fem_matrix_info              A_bsr.nnz / nrow                    solver.py:322-328
 *
 * Conventions.  All vectors are contiguous float32 [n, 3] (x, y, z per node), all
 * index arrays int32.  Pointers passed to fem_step / fem_refresh_tangent /
 * fem_eval_forces / fem_export_* are DEVICE pointers; FemDesc pointers are HOST
 * pointers that fem_create copies (the handle owns every device buffer it
 * allocates).  Every entry point enqueues work on the given CUDA stream
 * (cudaStream_t passed as void*; NULL = legacy default stream) and returns
 * without host synchronisation, except fem_create, fem_get_stats and
 * fem_matrix_info.  fem_step, fem_refresh_tangent (after its first call) and
 * fem_refresh_preconditioner allocate nothing and may be captured in a CUDA
 * graph.  A handle is not thread-safe; use one handle per stream.
 */
#ifndef FEM_GB300_H
#define FEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (int return of every entry point). */
#define FEM_OK 0
#define FEM_ERR_BAD_ARG 1      /* reference: ValueError */
#define FEM_ERR_NOT_CONVERGED 2 /* informational: CG hit maxiter above tolerance */
#define FEM_ERR_NON_FINITE 3    /* NaN/Inf in the solve */
#define FEM_ERR_TIMEOUT 4       /* a bounded device wait gave up (grid barrier) */
#define FEM_ERR_CUDA 5          /* CUDA runtime error */
#define FEM_ERR_UNSUPPORTED 6   /* option outside the implemented hot path */

/* Preconditioner kinds (SolverFEM preconditioner_type). */
#define FEM_PRECOND_BLOCK_DIAG 0 /* "block_diag": 3x3 block Jacobi, kernels.py:1817-1868 */
#define FEM_PRECOND_DIAG 1       /* "diag": point Jacobi of the scalar diagonal */

/* Force-term bits for fem_eval_forces (solver.py:571-582 order). */
#define FEM_TERM_SPRING 1
#define FEM_TERM_TET 2
#define FEM_TERM_HEX 4
#define FEM_TERM_GROUND 8
#define FEM_TERM_GRAVITY 16
#define FEM_TERM_DAMPING 32
#define FEM_TERM_TRI 64           /* triangle membrane, kernels.py:876-960 */
#define FEM_TERM_PARTICLE 128     /* hash-grid particle-particle contact, kernels.py:1036-1114 */
#define FEM_TERM_SOFT_CONTACT 256 /* soft-rigid contact list, kernels.py:1198-1261 */
#define FEM_TERM_SURFACE 512      /* soft-body surface contacts, soft_surface_contacts.py */
#define FEM_TERM_ALL 1023

typedef struct FemHandle FemHandle;

/* Construction data: Newton Model fields plus SolverFEM keyword arguments. */
typedef struct FemDesc {
    int32_t particle_count; /* P */
    int32_t tet_count;      /* T */
    int32_t hex_count;      /* H */
    int32_t spring_count;   /* S */
    const float* particle_q;        /* [P,3] construction positions (Dirichlet anchors, initial tangent) */
    const float* particle_mass;     /* [P] */
    const float* particle_inv_mass; /* [P] */
    const float* particle_radius;   /* [P] or NULL (= 0) */
    const int32_t* particle_flags;  /* [P] or NULL (= all ACTIVE); bit 0 = ACTIVE */
    const int32_t* tet_indices;     /* [T,4] */
    const float* tet_poses;         /* [T,3,3] row-major inverse rest edge matrices */
    const float* tet_materials;     /* [T,3] (mu, lambda, damping) */
    const int32_t* hex_indices;     /* [H,8] VTK order */
    const float* hex_materials;     /* [H,3] */
    const float* hex_inv_J0;        /* [H,8,3,3] */
    const float* hex_det_J0_w;      /* [H,8] */
    const int32_t* spring_indices;  /* [2S] */
    const float* spring_rest_length; /* [S] */
    const float* spring_stiffness;   /* [S] */
    const float* spring_damping;     /* [S] */
    const int32_t* fixed_indices;    /* [fixed_count] unique, in range */
    int32_t fixed_count;
    const int64_t* scene_offsets;    /* [scene_count+1] node ranges of independent scenes, NULL = one scene */
    int32_t scene_count;
    float gravity[3];          /* model gravity, used when fem_step gets no gravity pointer */
    float dt;                  /* assembly timestep */
    float min_stretch;         /* < 0 disables the clamp */
    float max_stretch;
    int32_t has_ground;
    float ground_plane[4];     /* n.x + d = 0 */
    float ground_ke, ground_kd, ground_kf, ground_mu;
    float linear_damping;
    int32_t enable_tet_activations;
    int32_t preconditioner;    /* FEM_PRECOND_* */
    int32_t maxiter;
    float tolerance;
    float* velocity_increment; /* optional caller-owned DEVICE [P,3] buffer for dv; NULL = handle-owned */
    /* Triangles (Newton tri_*): membrane + area + drag/lift force, lumped
     * constant tangent h^2 (mu + lambda) A_rest / 3 on each vertex diagonal. */
    int32_t tri_count;             /* Tri */
    const int32_t* tri_indices;    /* [Tri,3] */
    const float* tri_poses;        /* [Tri,2,2] inverse rest edge matrix in the triangle's own frame */
    const float* tri_materials;    /* [Tri,5] (ke, ka, kd, drag, lift) */
    /* Spring bend torque (solver.py:1437-1475): active when torque_stiffness > 0
     * and spring_rest_direction is given. */
    const float* spring_rest_direction; /* [S,3] unit rest directions or NULL */
    float torque_stiffness, torque_damping;
    /* Particle-particle self contact (solver.py:1477-1511): active when
     * particle_contact != 0 (ke > 0, P > 1, max radius > 0 and a grid). */
    int32_t particle_contact;
    float particle_ke, particle_kd, particle_kf, particle_mu, particle_cohesion, particle_max_radius;
    /* Soft-rigid contact material (Newton model.soft_contact_*); the contact
     * list itself is registered per step with fem_set_soft_contacts. */
    float soft_contact_ke, soft_contact_kd, soft_contact_kf, soft_contact_mu;
} FemDesc;

/* Per-solve statistics (one entry per scene, plus the sticky device status). */
typedef struct FemStats {
    int32_t status;        /* FEM_OK or FEM_ERR_TIMEOUT / FEM_ERR_NON_FINITE bits (sticky until fem_reset) */
    int32_t scene_count;
    int32_t max_iterations; /* maximum CG iterations over scenes in the last solve */
    int32_t min_iterations;
    float max_relative_residual; /* max over scenes of ||r||/||b|| (recurrence residual) */
    int32_t unconverged_scenes;
    int64_t total_iterations;    /* CG iterations summed over scenes and launches since creation */
} FemStats;

int fem_create(const FemDesc* desc, FemHandle** out);
int fem_destroy(FemHandle* handle);

/* One linearly implicit substep.  q_in / v_in are restored in place at fixed
 * nodes (reference semantics), f_workspace receives the final RHS
 * h*sum(f) - h^2 K v (projected), q_out / v_out the new state.
 * external_forces, activations and gravity may be NULL (gravity NULL = the
 * construction-time value; activations only with enable_tet_activations). */
int fem_step(FemHandle* handle, float* q_in, float* v_in, float* q_out, float* v_out, float* f_workspace,
             const float* external_forces, const float* activations, const float* gravity, float dt, void* stream);

/* Refresh the deformation-dependent tangent at q (fixed nodes restored in q
 * first) and the block-Jacobi inverse.  A changed dt also rebuilds the
 * mass/spring blocks and zeroes the warm start. */
int fem_refresh_tangent(FemHandle* handle, float* q, float dt, void* stream);
/* Rewrite only the Tet4/Hex8 blocks at q and dt (mass/spring blocks keep the
 * assembly dt), then the preconditioner. */
int fem_rebuild_element_blocks(FemHandle* handle, float* q, float dt, void* stream);
int fem_refresh_preconditioner(FemHandle* handle, void* stream);

int fem_set_tolerance(FemHandle* handle, float tolerance);
/* Time limit of every bounded device wait (grid barrier) in nanoseconds,
 * default 2e9.  A wait that runs out makes the kernel return early and sets the
 * sticky FEM_ERR_TIMEOUT status that fem_get_stats reports. */
int fem_set_wait_limit(FemHandle* handle, int64_t nanoseconds);

/* Launch tuning of the persistent PCG kernel (chosen by an autotuner).  Not
 * capturable: a change rebuilds the launch tables. */
#define FEM_TUNE_SPMV_UNROLL 1       /* block columns in flight per thread: 1, 2 or 4 (default 4) */
#define FEM_TUNE_L2_RESIDENT_BYTES 2 /* matrix bytes loaded evict_last (kept in L2 across iterations); -1 = 60% of L2;
                                        -2 (default) = the whole matrix when it fits in 60% of L2, else none */
#define FEM_TUNE_RESIDENT_SLICES 3   /* read-only: resulting number of L2-resident 32-row slices */
#define FEM_TUNE_GRID 4              /* read-only: cooperative grid size */
#define FEM_TUNE_CTA_THREADS 5       /* threads per PCG CTA: 256, 512, 1024, or 0 = automatic (default): one CTA with a
                                        warp per slice for at most 32 slices (no grid barriers), 1024 when there are
                                        at least 8 slices per SM (then at least one CTA per SM), else 256; the
                                        getter returns the size in use */
#define FEM_TUNE_GRID_CAP 6          /* upper bound on the PCG grid (0 = as many CTAs as fit, the default) */
#define FEM_TUNE_RESIDENT_STATE 7    /* read-only: the resident layout in use (0 none, 1 x/r/z, 2 x/r/z and the
                                        inverse diagonal blocks kept in each CTA's shared memory for the whole solve) */
#define FEM_TUNE_BALANCE 8           /* 1: split the rows over the PCG CTAs by each CTA's measured SpMV speed (a few
                                        10-iteration calibration solves, host-synchronous; results stay deterministic
                                        for the handle); 0 (default): split by stored blocks only */
#define FEM_TUNE_RESIDENT_LAYOUT 9   /* requested resident layout: -1 automatic (default), 0, 1 or 2 (see above); taken
                                        only when it costs no co-resident CTAs */
#define FEM_TUNE_SPLIT_HEADROOM 10   /* percent more slices than the even share a calibrated split may give one CTA
                                        (more shared memory per CTA); default 0 */
#define FEM_TUNE_TAIL_PREFETCH 11    /* when a CTA's second (last) round of slices keeps at most this percent of its
                                        warps busy, an idle warp requests that round's matrix bytes into L2 during the
                                        first round; 0 = off, default 50 */
#define FEM_TUNE_COMPACT_COLUMNS 12  /* column storage the PCG reads when every stored block's column - row offset fits
                                        16 bits: 0 32-bit columns; 1 16-bit offsets; 2 16-bit offsets, except at the
                                        slots where all 32 rows of a slice have the same offset, which are read once
                                        per slice from shared memory; -1 (default) automatic: 2 when the matrix
                                        streams from DRAM, 1 when all of it is kept in L2.  The getter returns the mode
                                        in use (0 when the offsets do not fit) */
#define FEM_TUNE_UNIFORM_COLUMN_BLOCKS 13  /* read-only: stored blocks whose column offset mode 2 reads once per slice */
#define FEM_TUNE_CG_VARIANT 14       /* CG recurrence of the persistent PCG: 0 standard (two grid reductions per
                                        iteration); 1 Chronopoulos-Gear (one reduction per iteration; neighbours'
                                        next preconditioned residual recomputed at every gathered column) */
#define FEM_TUNE_OPERATOR_BATCH 15   /* fem_apply_operator: block columns loaded before any is used, per thread: 2 at
                                        32 registers (8 CTAs of 256 threads per SM, the default: a 64^3 Hex8 matrix in
                                        one wave, 51 us) or 4 at 48 registers (5 CTAs per SM: 1.4 waves, 63 us) */
#define FEM_TUNE_OPERATOR_STAGE 16   /* fem_apply_operator: 4 (default) or 8 stages the block planes through shared
                                        memory with bulk asynchronous copies (cp.async.bulk), that many block columns
                                        of a slice per copy, double-buffered per warp (64^3 Hex8: 49 us with 4, 74 us
                                        with 8); 0 loads them directly (FEM_TUNE_OPERATOR_BATCH applies).  Staging
                                        needs the 16-bit column offsets (FEM_TUNE_COMPACT_COLUMNS not 0); otherwise
                                        the direct loads run.  A copy that does not complete within the wait limit
                                        sets the timeout status that fem_get_stats reports. */
int fem_set_tuning(FemHandle* handle, int32_t key, int64_t value);
int fem_get_tuning(FemHandle* handle, int32_t key, int64_t* value);
int fem_set_maxiter(FemHandle* handle, int32_t maxiter);
int fem_reset(FemHandle* handle, void* stream);
float* fem_velocity_increment_ptr(FemHandle* handle);
/* Largest final relative residual ||r|| / ||b|| of the handle's solves since
 * the last reset: residuals[0] over step-mode solves (fem_step, rollouts),
 * residuals[1] over solve-mode solves (fem_solve, adjoint solves); a
 * non-finite residual reads 1e30.  Synchronises the stream; reset != 0 clears
 * both.  Backs SolverFEM.check() of the differentiable mode (the reference's
 * differentiation.check, differentiation.py:263-272, with its deferred checks). */
int fem_get_solve_residuals(FemHandle* handle, float* residuals, int32_t reset, void* stream);
int fem_get_stats(FemHandle* handle, FemStats* stats, int32_t* scene_iterations, void* stream);

/* Measurement support: when enabled, every eager (not graph-captured)
 * fem_step brackets its PCG launch with CUDA events on the launch stream;
 * fem_get_timing synchronises, returns the summed launch time and count, and
 * clears the record. */
int fem_set_timing(FemHandle* handle, int32_t enable);
int fem_get_timing(FemHandle* handle, double* pcg_ms_total, int64_t* launches);

/* Soft-rigid contacts for the following fem_step / fem_eval_forces / fem_prepare
 * calls (SolverFEM.eval_soft_contact_forces, solver.py:1540-1566, over Newton's
 * Contacts.soft_contact_*).  Device pointers: count [1] (read on the device, so
 * no host sync), particle [capacity], body_pos / body_vel / normal
 * [capacity,3]; entries at or past *count, or with a particle outside [0, P),
 * are ignored.  capacity 0 (or NULL pointers) clears the registration.  A
 * larger capacity than before allocates scratch, so register before capture. */
int fem_set_soft_contacts(FemHandle* handle, const int32_t* count, const int32_t* particle, const float* body_pos,
                          const float* body_vel, const float* normal, int32_t capacity);

/* Soft-body surface contacts (SolverFEM.set_soft_surface_contacts, solver.py:510-540;
 * soft_surface_contacts.py).  body_count bodies, body b owning particles
 * [body_start[b], body_start[b] + body_size[b]) and the surface triangles
 * triangles[tri_offsets[b] .. tri_offsets[b+1]) (3 local indices each; HOST
 * arrays).  Each surface vertex feels the other bodies' surfaces within their
 * rest bounding-box diagonal: penetration r - signed distance (sign from the
 * angle-weighted pseudonormal), force n (ke pen - kd min(v.n, 0)).  The
 * surfaces take the positions q (DEVICE [P,3]) now and at every refit.
 * body_count 0 clears the registration.  Allocates: call before capture. */
int fem_set_surface_contacts(FemHandle* handle, int32_t body_count, const int32_t* body_start, const int32_t* body_size,
                             const int32_t* tri_offsets, const int32_t* triangles, float ke, float kd, const float* q,
                             void* stream);
/* Refit the registered surfaces at q (SoftBodySurfaceContacts.update); also
 * done by the first fem_refresh_tangent and by fem_rebuild_element_blocks. */
int fem_update_surface_contacts(FemHandle* handle, const float* q, void* stream);

/* Selected force terms (FEM_TERM_* bits), unscaled, summed into out[P,3]. */
int fem_eval_forces(FemHandle* handle, const float* q, const float* v, const float* activations,
                    const float* gravity, int32_t terms, float* out, void* stream);

/* Sparse matrix in the reference's BSR form: offsets [P+1], columns [nnzb],
 * values [nnzb,3,3]; any pointer may be NULL. */
int fem_matrix_info(FemHandle* handle, int64_t* nnzb, int64_t* triplet_count, int64_t* stored_blocks);
int fem_export_bsr(FemHandle* handle, int32_t* offsets, int32_t* columns, float* values, void* stream);
int fem_export_preconditioner(FemHandle* handle, float* inverse_blocks, void* stream);
/* Raw element/constant blocks in the reference's triplet layout [P | 2S | 3Tri | 16T | 64H] (bsr_values). */
int fem_export_triplets(FemHandle* handle, int32_t* rows, int32_t* columns, float* values, void* stream);

/* ---- Differentiation with the system matrix held fixed (the reference's
 * differentiable branch, differentiation.py:149-394).  A substep is
 * rhs = h sum f(q, v, a) + h ext - sum_j A_ij (v_j - v_i) + spring damping,
 * dv = (PAP + I - P)^-1 P rhs, v' = v + dv, q' = q + h v'.  Its VJP uses a
 * second solve with the same symmetric A (fem_solve), the force VJP
 * (fem_force_vjp) and the predictor VJP (fem_predictor_vjp). */

/* Optional per-tet shear scale (device [T], NULL to clear) multiplying mu in
 * the force and tangent kernels; the pointer is read at every launch.  Beyond
 * the reference (its differentiable controls are the additive activations). */
int fem_set_mu_scale(FemHandle* handle, const float* scale);
/* Solve (PAP + I - P) x = P rhs from x = 0 to ||r|| <= tolerance ||P rhs||
 * (at most maxiter iterations) with the reference's RHS normalisation. */
int fem_solve(FemHandle* handle, const float* rhs, float* x, float tolerance, int32_t maxiter, void* stream);
/* Accumulate (d sum f / d q)^T force_bar into q_bar and (d sum f / d v)^T
 * force_bar into v_bar over all force terms at (q, v, activations); write
 * dL/d activation and dL/d mu_scale per tet when those pointers are given.
 * The first call allocates adjoint scratch (call it once before capture). */
int fem_force_vjp(FemHandle* handle, const float* q, const float* v, const float* activations, const float* gravity,
                  const float* force_bar, float* q_bar, float* v_bar, float* activation_bar, float* mu_scale_bar,
                  void* stream);
/* Accumulate the predictor's VJP into v_bar: -(A rhs_bar)_k + (sum_j A_kj)^T rhs_bar_k
 * plus the spring-damping term (implicit_predictor.py:9-41). */
int fem_predictor_vjp(FemHandle* handle, const float* rhs_bar, float dt, float* v_bar, void* stream);
/* fem_force_vjp plus the gradient wrt each element's raw material row (the
 * force kernels' inputs, kernels.py:541-581 for Tet4 and 1481-1601 for Hex8):
 * tet_material_bar [T,3] and hex_material_bar [H,3] receive dL/d(mu, lambda,
 * k_d); either may be NULL.  Beyond the reference, whose differentiable mode
 * holds materials fixed (differentiation.py:254-276); the matrix stays fixed
 * at its assembly materials, as for every differentiable input. */
int fem_force_vjp_materials(FemHandle* handle, const float* q, const float* v, const float* activations,
                            const float* gravity, const float* force_bar, float* q_bar, float* v_bar,
                            float* activation_bar, float* mu_scale_bar, float* tet_material_bar,
                            float* hex_material_bar, void* stream);

/* Device-side differentiable rollouts over the fixed matrix: whole segments of
 * substeps enqueued from C++ on one stream, with no host synchronisation, in
 * place of the reference's taped per-substep Python (differentiation.step,
 * differentiation.py:287-394, driven per substep by the bear-training loop's
 * frame checkpoints, examples/diffsim/_bear_training.py:239-310).
 *
 * fem_rollout_segment: `substeps` differentiable substeps from (q0, v0),
 * writing the states before and after every substep into q_states / v_states
 * ([substeps+1, P, 3]; q0 / v0 may already be slot 0).  Each substep is
 * SolverFEM.step on the fixed matrix at (tolerance, maxiter).  warm_start 0:
 * every solve starts from zero (the reference's checked solves); 1: the first
 * from dv0 (NULL = zero), the rest from the previous increment, and the last
 * increment goes to dv_out (optional).  refresh != 0 first assembles the
 * tangent at q0, so a segment can be one frame of a frame loop.
 *
 * fem_adjoint_segment: the reverse pass over such a segment.  q_bar, v_bar
 * [P,3] hold dL/d(state after the last substep) on entry and dL/d(state
 * before the first) on return.  Per substep, in reverse: the adjoint solve
 * with the same symmetric matrix, the predictor VJP and the force VJP.
 * Accumulated (+=) when given: ext_bar [P,3] (a load held over the segment),
 * activation_bar / mu_scale_bar [T], tet_material_bar [T,3], hex_material_bar
 * [H,3].  adjoint_start [P,3] (optional) is the warm start of each adjoint solve
 * and receives its solution (NULL = every adjoint solve from zero).  refresh
 * != 0 first assembles the tangent at q_states[0] (the matrix the segment's
 * forward used when it was rolled out with refresh).  dt must equal the
 * assembled timestep.  The first call allocates scratch: call once before
 * capturing either function in a CUDA graph. */
int fem_rollout_segment(FemHandle* handle, const float* q0, const float* v0, const float* dv0, int32_t substeps,
                        const float* external_forces, const float* activations, const float* gravity, float dt,
                        float tolerance, int32_t maxiter, int32_t warm_start, int32_t refresh, float* q_states,
                        float* v_states, float* dv_out, void* stream);
int fem_adjoint_segment(FemHandle* handle, float* q_states, float* v_states, int32_t substeps,
                        const float* external_forces, const float* activations, const float* gravity, float dt,
                        float tolerance, int32_t maxiter, int32_t refresh, float* adjoint_start, float* q_bar,
                        float* v_bar, float* ext_bar, float* activation_bar, float* mu_scale_bar,
                        float* tet_material_bar, float* hex_material_bar, void* stream);

/* Rebuild the constant matrix, the sparsity pattern, the slot map and the
 * preconditioner after in-place edits of tet connectivity, poses, materials
 * and masses (refresh_topology, solver.py:872-940; the sorted path, without
 * streaming assembly).  d describes the model's current arrays with the same
 * counts, scenes and fixed set as at creation; dt must equal the assembled
 * timestep.  The tangent is then assembled at q (fixed nodes restored in
 * place) and the velocity increment is cleared.  The handle's internal
 * storage is rebuilt, so graphs captured before the call must be captured
 * again. */
int fem_refresh_topology(FemHandle* h, const FemDesc* d, float* q, float dt, void* stream);

/* ---------------------------------------------------------------------------
 * Streaming Tet4 assembly (streaming.py, StreamingTetAssembly;
 * SolverFEM.prepare_tetrahedral_updates solver.py:693-719, refresh_topology
 * with element_sources solver.py:872-940).  The particle pool holds equal
 * copies of N0 original nodes (pool node i represents original node i % N0);
 * tetrahedra may move their corners onto any copy of their original corners.
 * Requires Tet4 elements only, block_diag, no fixed nodes and one scene.
 * ------------------------------------------------------------------------- */
typedef struct FemTopologyUpdate {
    int32_t dirty_elements;             /* active elements whose blocks changed */
    int32_t removed_elements;           /* previous elements whose contribution was withdrawn */
    int32_t reused_elements;            /* unchanged connectivity, positions, pose and material */
    int32_t active_elements;
    int32_t touched_rows;               /* rows whose sparse structure changed */
    int32_t topology_inserted_elements;
    int32_t topology_removed_elements;
    int32_t full_numeric_refresh;       /* more than half the active elements were dirty */
} FemTopologyUpdate;

/* Reserve the candidate pattern (row r: r and every copy of every original
 * neighbour of r mod N0 over the enabled tets of d) and assemble at the
 * construction positions.  Rebuilds the handle's storage once; call before
 * capturing graphs.  d describes the model's arrays as at creation. */
int fem_prepare_tet_updates(FemHandle* h, const FemDesc* d, int32_t original_node_count, void* stream);
/* Apply edited tet connectivity, poses, materials, masses and flags (from d)
 * at positions q without moving any device storage: a graph captured before
 * the call replays after it.  element_sources (device int32 [T], or NULL for
 * the identity) gives each slot's previous element or -1.  Validation runs
 * before any change; a rejected update returns FEM_ERR_BAD_ARG and leaves the
 * assembly untouched.  Clears the warm start; synchronises the stream. */
int fem_update_tet_topology(FemHandle* h, const FemDesc* d, float* q, float dt, const int32_t* element_sources,
                            FemTopologyUpdate* update, void* stream);

/* ---------------------------------------------------------------------------
 * Prepared affine step.  Replaces the reference's PreparedFEMStep
 * (prepared_step.py:64-302; SolverFEM.prepare_step, solver.py:483-500).  The
 * caller owns the workspace: seven device arrays, [N,3] float32 except
 * diagonal ([N,3,3]); the functions read and write only those and the
 * handle's matrix, preconditioner and scratch.
 * ------------------------------------------------------------------------- */
typedef struct FemPreparedWs {
    float* q;          /* prepared positions (fixed nodes restored) */
    float* v;          /* prepared velocities (fixed nodes zero) */
    float* impulse;    /* h * sum of the force terms (+ h * the load passed to fem_prepare) */
    float* predictor;  /* sum_j A_ij (v_j - v_i) */
    float* base_rhs;   /* fem_prepared_rhs with no extra load */
    float* increment;  /* the workspace's velocity increment (warm start of fem_prepared_solve) */
    float* diagonal;   /* diagonal blocks of PAP + I - P (identity at fixed nodes) */
} FemPreparedWs;

/* prepared_step.py:126-183: copies q_in, v_in (unchanged), evaluates the force terms once. */
int fem_prepare(FemHandle* h, const FemPreparedWs* ws, const float* q_in, const float* v_in,
                const float* external_forces_or_null, const float* activations_or_null, const float* gravity,
                float dt, void* stream);
/* prepared_step.py:185-213: out = impulse + dt*ext - predictor + spring damping, zero at fixed nodes.
 * out must not alias ext. */
int fem_prepared_rhs(FemHandle* h, const FemPreparedWs* ws, const float* external_forces_or_null, float dt, float* out,
                     void* stream);
/* prepared_step.py:215-224: y = (PAP + I - P) x; x and y distinct. */
int fem_apply_operator(FemHandle* h, const float* x, float* y, void* stream);
/* prepared_step.py:226-235: z = M r (block-Jacobi, or point-Jacobi with preconditioner=1); r and z distinct. */
int fem_apply_preconditioner(FemHandle* h, const float* r, float* z, void* stream);
/* prepared_step.py:252-275: normalised PCG for (PAP + I - P) dv = rhs from ws->increment; the result
 * replaces ws->increment.  Statistics through fem_get_stats. */
int fem_prepared_solve(FemHandle* h, const FemPreparedWs* ws, const float* rhs, float tolerance, int32_t maxiter,
                       float dt, void* stream);
/* prepared_step.py:277-302: v_out = ws->v + dv, q_out = ws->q + dt * v_out, fixed nodes restored;
 * the outputs must not be the workspace arrays. */
int fem_prepared_reconstruct(FemHandle* h, const FemPreparedWs* ws, const float* dv, float dt, float* q_out,
                             float* v_out, void* stream);

/* Block-Jacobi PCG on a caller-supplied BSR matrix that allocates no device
 * memory.  No counterpart in the reference: it exists for callers that cannot
 * call cudaMalloc at solve time (a host application that owns all device
 * memory or forbids runtime allocations, or a real-time loop that cannot take
 * an allocation's implicit synchronisation), which rules out fem_create.
 * offsets [rows+1], columns [nnzb], values [nnzb,3,3], rhs [rows,3] and
 * x_inout [rows,3] (warm start in, solution out) are device pointers; info is
 * an optional device int[2] receiving (iterations, status bits: 1 a bounded
 * grid-barrier wait timed out, 2 a non-finite value).  Solves A x = rhs to
 * ||r|| <= tolerance ||rhs|| with the reference's RHS normalisation and at
 * most maxiter iterations.  There is no fixed-node projection: the caller's
 * matrix and rhs must already hold it (identity rows and zero columns at
 * fixed nodes, zero rhs there), as SolverFEM's exported operator does.
 * Failures are reported only on the device: the return code covers argument
 * and launch errors, so with info == NULL a timeout or a non-finite solve goes
 * unnoticed.  After a non-finite solve x_inout keeps the warm start; after a
 * timeout its contents are unspecified.  Each wait gives up after 2 s, or after
 * the nanoseconds in the environment variable FEM_NOALLOC_WAIT_LIMIT_NS (read
 * at every call).  Working vectors live in a static device array sized for at
 * most 65,536 block rows (about 6.5 MB per GPU that loads the library, held
 * until exit); larger systems return FEM_ERR_BAD_ARG.  The first call on a
 * device resolves that array's address and must come before any stream
 * capture; calls after cudaDeviceReset are not supported.  All calls share the
 * array, so calls that overlap on the GPU race; serialise them. */
int fem_pcg_solve_noalloc(const int32_t* offsets, const int32_t* columns, const float* values, const float* rhs,
                          float* x_inout, int32_t rows, float tolerance, int32_t maxiter, int32_t* info,
                          void* stream);

const char* fem_status_string(int status);
const char* fem_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FEM_GB300_H */
