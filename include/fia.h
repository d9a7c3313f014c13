/*
 * fia.h -- C ABI of the GB300 flux-interpolated advection library (libfia.so).
 *
 * The library replaces the 3D hot path of the reference program
 * (nyhirasawa/Flux-Interpolated-Advection): the density flux advection
 * (move_substances_3D), the velocity flux advection
 * (advect_velocity_xyz_flux_advection_3D_std_thread), the pressure projection
 * (calc_pressure_3D / calc_pressure_gradient_term_3D) and the CFL time step.
 * Only plain C types cross this boundary; fields use the reference's Grid_3D layout
 * (grid_3d.h:35-54): z fastest, x slowest; density and pressure nx*ny*nz, u (nx+1)*ny*nz,
 * v nx*(ny+1)*nz, w nx*ny*(nz+1); cell length h, domain [0, n*h]^3, closed box.
 *
 * Errors: every function returns FIA_OK (0) or a negative FIA_ERR_* code; a positive
 * return is a set of FIA_STATUS_* bits (the call completed, with numerical warnings).
 * The reference itself has no error convention (void functions, exit(0) in the face
 * clipper at facecutter.h:191-204); the C++ shim with the reference's void signatures
 * (fia_shim.hpp in the library's shim directory) exits on an error code.
 */
#ifndef FIA_H
#define FIA_H

#ifdef __cplusplus
extern "C" {
#endif

#define FIA_API_VERSION 1

/* return codes */
#define FIA_OK 0
#define FIA_ERR_INVALID -1      /* bad argument (null pointer, size, enum value) */
#define FIA_ERR_CUDA -2         /* a CUDA call failed (fia_error_string has the text) */
#define FIA_ERR_UNSUPPORTED -3  /* option the library does not implement */
#define FIA_ERR_NOMEM -4        /* device allocation failed */

/* status bits (positive returns, also fia_last_status) */
#define FIA_STATUS_CLIP_OVERFLOW 1    /* a clipped piece exceeded 32 vertices (MAX_TMP_POINTS), or in
                                         the FP32C form a face produced more than 128 pieces */
#define FIA_STATUS_CLIP_ODD_CUT 2     /* odd number of iso-line crossings; the reference exit(0)s */
#define FIA_STATUS_NONFINITE 4        /* a non-finite face flux was produced */
#define FIA_STATUS_SUBDIV_OVERFLOW 8  /* minimal_area triangulation stack exhausted */
#define FIA_STATUS_SOLVER_CAP 16      /* pressure solver stopped at max_iter before tol */
#define FIA_STATUS_SOLVER_FALLBACK 32 /* learned-preconditioned FCG fell back to plain PCG */

/* device precision of a session */
#define FIA_FP64 0   /* plain form: FP64 throughout */
#define FIA_FP32C 1  /* chosen form: FP32 advection with compensated sums, FP64 reductions */

/* element type of host buffers */
#define FIA_HOST_F64 0
#define FIA_HOST_F32 1

/* fields */
#define FIA_FIELD_DENSITY 0
#define FIA_FIELD_U 1
#define FIA_FIELD_V 2
#define FIA_FIELD_W 3
#define FIA_FIELD_PRESSURE 4

/* interpolation_method (main.cpp:60) */
#define FIA_INTERP_WENO6 0
#define FIA_INTERP_LINEAR 1

/* split_method (split_face_3D.cpp:26-41); the density main pass uses the caller's */
#define FIA_SPLIT_XZ_CELLFACE 0           /* "xz-CellFaceAligned" */
#define FIA_SPLIT_XZ_AXIS 1               /* "xz-AxisAligned" */
#define FIA_SPLIT_XCELLFACE_ZAXIS 2       /* "x-CellFaceAligned_z-AxisAligned" */
#define FIA_SPLIT_XAXIS_ZCELLFACE 3       /* "x-AxisAligned_z-CellFaceAligned" */

/* pressure solvers */
#define FIA_SOLVER_PCG_JACOBI 0
#define FIA_SOLVER_FCG_LEARNED 1   /* flexible CG around the learned two-level preconditioner (FP32C
                                      sessions); Jacobi-PCG takes over after fallback_iter iterations */

typedef struct fia_session fia_session;

/* Flags of move_substances_3D / advect_velocity_xyz_flux_advection_3D_std_thread
 * (move_substances_3d.h:48-66, advect_velocity_flux_advection_3d.h:107-124), same names. */
typedef struct fia_advect_params {
    int interpolation_method;                               /* FIA_INTERP_* */
    int split_method;                                       /* FIA_SPLIT_*, density main pass */
    int num_gauss_quadrature_point_for_integrate_density;   /* odd, 1..15 */
    int use_integral;                                       /* y-integral quadrature (main.cpp:64) */
    int enable_eliminate_zero_velocity_false_diffusion;     /* passes 2 and 3 (main.cpp:70) */
    int use_MacCormack_scheme;                              /* flux MacCormack: each face at rest, backtraced
                                                               and traced back, weights 0.5, 1, -0.5
                                                               (backtrace_..._for_integrate_density.cpp:146-234);
                                                               not in fia_move_substances_3D_noalloc */
    int enable_cell_volume_correction;                      /* density: cell volumes from the pieces'
                                                               y n_y, Poisson solve of -(V - V0), mass
                                                               exchanged between neighbours
                                                               (move_substances_3d.cpp:243-493); both
                                                               forms (FIA_ERR_UNSUPPORTED in the
                                                               allocation-free entry point) */
    double minimal_area;                                    /* xi-eta triangulation threshold (main.cpp:82);
                                                               below 1 (triangulated pieces) the FP64 form
                                                               only: FIA_ERR_UNSUPPORTED in FP32C */
} fia_advect_params;

typedef struct fia_solver_params {
    double tol;        /* relative residual |b - A p| / |b| */
    int max_iter;
    int method;        /* FIA_SOLVER_* */
    int fallback_iter; /* FIA_SOLVER_FCG_LEARNED: FCG iterations before the Jacobi-PCG fallback */
} fia_solver_params;

typedef struct fia_solver_report {
    int iterations;    /* all iterations (FCG + fallback PCG) */
    double rel_residual;
    int status;        /* FIA_STATUS_* bits of the solve */
    int fcg_iterations;        /* of which flexible-CG iterations with the learned preconditioner */
    double precond_ms;         /* device time in the preconditioner (0 unless profiled) */
} fia_solver_report;

/* One smoke step in the order of the reference's 3D loop (main.cpp:600-721): CFL time
 * step, body force, velocity update (frame 0: project then advect, afterwards advect then
 * project; update_fluid_velocity_3d.cpp:116-192), density advection.  The plume source,
 * the buoyancy force and the mass correction have no counterpart in the reference
 * (add_force_fluid_3D is commented out at update_fluid_velocity_3d.cpp:109 and
 * correct_volume_concentration_error.cpp is empty); they are off when zero. */
typedef struct fia_step_params {
    fia_advect_params advect;     /* density and velocity flux advection */
    fia_solver_params solver;     /* pressure projection */
    double cfl;                   /* dt = cfl * h / max|u|   (calc_time_step_length_from_CFL_number.cpp:119) */
    double max_dt;                /* cap on dt (the reference caps at the next movie frame, 1/fps) */
    double buoyancy;              /* upward acceleration per unit density, added to v before advection */
    int source;                   /* re-inject density in a sphere at the start of the step */
    double source_center[3];
    double source_radius;
    double source_density;
    int mass_correction;          /* rescale density to its pre-advection mass (FP64 sums) */
    int frame;                    /* step index i_frame */
    int capture_pair;             /* before the projection, solve it to capture_tol with Jacobi-PCG and
                                     keep (rhs, pressure) as a training pair of the learned preconditioner */
    double capture_tol;
} fia_step_params;

typedef struct fia_step_report {
    double dt;
    double max_velocity;
    double mass_before_advection;
    double mass_after_advection;  /* before the mass correction */
    double mass_after;            /* after it */
    int solver_iterations;
    double solver_rel_residual;
    int status;                   /* FIA_STATUS_* bits of the step */
    int solver_fcg_iterations;    /* flexible-CG iterations of the learned solver */
    double precond_ms;            /* device time in the learned preconditioner */
} fia_step_report;

/* The Gauss rule of the y-integral quadrature for k points per half cell (odd, 1..15; k = 1
 * is the reference's default, main.cpp:69): nodes on [-1, 1] centre first, then -/+ pairs by
 * increasing |x| (the order of gauss_quadrature_points.cpp:18-60), weights normalised to sum
 * 1.  Host only (no device call). */
int fia_gauss_rule(int k, double* nodes, double* weights);

/* Reference defaults for the flags (main.cpp:48-83) with WENO6, xz-CellFaceAligned, k = 3. */
void fia_default_advect_params(fia_advect_params* p);
void fia_default_solver_params(fia_solver_params* p);
/* The plume of the benchmark configurations: source r = 0.1 at (0.5, 0.15, 0.5) of the unit
 * box, density 1, buoyancy 1, CFL 1, mass correction on. */
void fia_default_step_params(fia_step_params* p);
int fia_step(fia_session* s, const fia_step_params* p, fia_step_report* rep);

int fia_api_version(void);
const char* fia_error_string(int code);

/* Session: device-resident Grid_3D of nx*ny*nz cells (replaces the Grid_3D ctor,
 * grid_3d.cpp:13-47).  Returns NULL on failure.  Besides the fields it holds the store of a
 * pass's clipped pieces, sized for 10 pieces per node of the largest field at creation
 * (16 + 8 bytes a piece in the FP32C form, 40 in the FP64 form) and grown when a pass needs
 * more. */
fia_session* fia_create(int nx, int ny, int nz, double cell_length, int precision);
void fia_destroy(fia_session* s);
int fia_last_status(const fia_session* s);
/* The session's CUDA stream (a cudaStream_t), for callers that order their own work. */
void* fia_stream(fia_session* s);
int fia_synchronize(fia_session* s);

/* Host <-> device copies of one field (host_dtype FIA_HOST_F64 or FIA_HOST_F32). */
int fia_set_field(fia_session* s, int field, const void* host, int host_dtype);
int fia_get_field(fia_session* s, int field, void* host, int host_dtype);
/* Device address of a field (element type is the session precision's). */
int fia_field_device_ptr(fia_session* s, int field, void** dev_ptr);

/* move_substances_3D (move_substances_3d.cpp:38-240), flux branch, on the device. */
int fia_move_substances_3D(fia_session* s, double time_step_length, const fia_advect_params* p);
/* advect_velocity_xyz_flux_advection_3D_std_thread (advect_velocity_flux_advection_3d.cpp:1138-1272). */
int fia_advect_velocity_xyz(fia_session* s, double time_step_length, const fia_advect_params* p);
/* calc_pressure_3D (calc_pressure_3d.cpp:18-181): pressure of the current velocity. */
int fia_calc_pressure_3D(fia_session* s, const fia_solver_params* sp, fia_solver_report* rep);
/* calc_pressure_gradient_term_3D (calc_pressure_3d.cpp:183-270): solve, subtract, wall tallies. */
int fia_calc_pressure_gradient_term_3D(fia_session* s, const fia_solver_params* sp, fia_solver_report* rep);
/* The CFL reduction of calc_time_step_length_from_CFL_number_3D (:90-117). */
int fia_max_abs_velocity(fia_session* s, double* out);
/* Sum of density * cell volume (the mass of main.cpp:520-531), FP64. */
int fia_total_mass(fia_session* s, double* out);
/* total_loss_of_momentum_{x,y,z} accumulated by calc_pressure_gradient_term_3D. */
int fia_wall_momentum_loss(fia_session* s, double* out3);
/* Sum of face velocity * cell volume per component (the momenta of main.cpp:533-585), FP64. */
int fia_total_momentum(fia_session* s, double* out3);

/* Frame output of the reference's main loop (main.cpp:515-654).  The density frame the
 * reference exports as an OpenVDB grid (vdbexport.cpp:43-98: origin -L/2 per axis, voxel size
 * = cell length) is written as a dense little-endian file: the 64-byte header
 * fia_frame_header, then nx*ny*nz float32 values in the grid's linear order (z fastest). */
typedef struct fia_frame_header {
    char magic[8];        /* "FIAFRM1" and a zero byte */
    int nx, ny, nz;
    int frame;            /* movie frame index (the %04d of substance_density_%04d.vdb) */
    double origin[3];     /* world position of voxel (0,0,0)'s corner: -0.5 * cell length * n */
    double voxel_size;    /* cell length */
    int reserved[2];      /* zero */
} fia_frame_header;
int fia_write_density_frame(fia_session* s, const char* path, int frame);
/* Appends one "time value" line (16 significant digits) to each of the reference's logs under
 * the path prefix: total_mass.dat, total_momentum_{x,y,z}.dat, total_loss_of_momentum_{x,y,z}.dat
 * and momentum_{x,y,z}_plus_total_loss_of_momentum_{x,y,z}.dat. */
int fia_append_totals(fia_session* s, const char* prefix, double now_time);
/* Work counters accumulated since fia_create: [0] faces visited, [1] pieces emitted,
 * [2] faces clipped from both sides (an iso-line crossed a piece more than twice, so the
 * two adjacent cells see different pieces; FP32 form only counts [3]), [3] point
 * interpolations made by the FP32 face kernel, [4] kernels launched. */
int fia_pass_counters(fia_session* s, unsigned long long* out5);

/* Face-kernel timing: after fia_profile_faces(s, capacity) an event pair is recorded on the
 * session stream around each face-kernel launch (up to capacity launches);
 * fia_profile_faces_read returns their summed device time and count, and stops. */
int fia_profile_faces(fia_session* s, int capacity);
int fia_profile_faces_read(fia_session* s, double* total_ms, int* launches);

/* Drop-in bodies with host buffers: copy in, run on the device, copy out (synchronous). */
int fia_move_substances_3D_host(fia_session* s, int host_dtype, void* substance_density, const void* u,
                                const void* v, const void* w, double time_step_length,
                                const fia_advect_params* p);
int fia_advect_velocity_xyz_host(fia_session* s, int host_dtype, void* u, void* v, void* w,
                                 double time_step_length, const fia_advect_params* p);
int fia_calc_pressure_gradient_term_3D_host(fia_session* s, int host_dtype, void* u, void* v, void* w,
                                            void* pressure, const fia_solver_params* sp,
                                            fia_solver_report* rep);

/* move_substances_3D (FP64 plain form) on caller-owned DEVICE buffers, allocating nothing.
 * No counterpart in the reference.  For callers that cannot call cudaMalloc: a host
 * application that owns all device memory and hands a plug-in only the buffers it may touch
 * (a renderer or engine integration with a fixed memory budget), or a real-time loop where
 * an allocation's latency and possible failure are not acceptable.  The scratch of the pass
 * lives in a static device array of 23.6 MB that every GPU loading the library holds until
 * the process exits; grids are limited to 64 cells per axis (larger grids return
 * FIA_ERR_INVALID; fia_noalloc_error_string says why).  density_in and density_out must be
 * distinct; stream is a cudaStream_t (NULL: the legacy default stream); the call returns
 * after the pass has finished, with FIA_STATUS_* bits or an error code.  The first call on a
 * device looks up the scratch's device address (cudaGetSymbolAddress), and with CUDA's default
 * lazy module loading that is also when the driver reserves the 23.6 MB there: make one call
 * at initialisation (or set CUDA_MODULE_LOADING=EAGER), before any stream capture.  The
 * address is kept for the process's lifetime (no cudaDeviceReset after the first call).
 * All calls share the one scratch array: calls that overlap on the GPU (other streams or
 * host threads) race on it. */
int fia_move_substances_3D_noalloc(int nx, int ny, int nz, double cell_length, const double* density_in,
                                   double* density_out, const double* u, const double* v, const double* w,
                                   double time_step_length, const fia_advect_params* p, void* stream);
const char* fia_noalloc_error_string(void);

/* Solid spheres (no counterpart in the reference, whose 3D scenes have only the box walls):
 * cells whose centre lies inside a sphere are solid.  The projection treats them like walls
 * (zero-flux faces, the pressure unknowns removed; if the pinned last cell is solid the last
 * fluid cell is pinned instead), faces touching a solid cell get zero velocity, and density
 * is neither injected into nor kept in solid cells.  centers: 3*count doubles (physical
 * coordinates, origin at the box corner); count 0 removes all solids. */
int fia_set_solid_spheres(fia_session* s, int count, const double* centers, const double* radii);
/* the solid mask (1 byte per cell, reference cell order) */
int fia_get_solid_mask(fia_session* s, unsigned char* out);

/* Learned pressure preconditioner (no counterpart in the reference, which uses amgcl):
 * z = omega D^-1 r + P net(R r) with a 3D U-Net of 4 levels (16/32/48/64 channels,
 * 3x3x3 convolutions, BF16 weights, FP32 accumulation) on the half-resolution grid, used by
 * FIA_SOLVER_FCG_LEARNED.  The weights are one float array of fia_learned_num_parameters()
 * values: each layer's [tap][in][out] block in layer order, then omega. */
long long fia_learned_num_parameters(void);
int fia_learned_init(fia_session* s, unsigned long long seed);
int fia_learned_set_weights(fia_session* s, const float* w, long long count);
int fia_learned_get_weights(fia_session* s, float* w, long long count);
/* Training pairs B p = r (B = -A, r = -div(u) h) kept on the device, normalised to rms(r) = 1:
 * from host arrays of nx*ny*nz floats, or captured by fia_step (capture_pair). */
int fia_learned_add_pair(fia_session* s, const float* r, const float* p);
int fia_learned_num_pairs(fia_session* s);
/* Energy-norm loss (z - p)^T B (z - p) / p^T B p of the preconditioner on pair i. */
int fia_learned_loss(fia_session* s, int pair, double* loss);
/* Scales the output layer so that the preconditioner's output best fits pair i (least squares
 * in the energy norm); used once after fia_learned_init. */
int fia_learned_calibrate(fia_session* s, int pair);
/* One Adam step on the mean gradient over pairs[0..batch); losses[i] receives each pair's loss. */
int fia_learned_train_step(fia_session* s, const int* pairs, int batch, double lr, double* losses);
/* Network dimensions: level 0 .. 3 grid sizes (dims3 out). */
int fia_learned_level_dims(fia_session* s, int level, int* dims3);
/* Test hooks: the network alone on a level-0 scalar input (host floats, level-0 size),
 * its gradient with respect to all parameters for a given dL/dy (host floats), and the
 * preconditioner applied to a fine-grid residual. */
int fia_debug_unet_forward(fia_session* s, const float* x0, float* y);
int fia_debug_unet_backward(fia_session* s, const float* x0, const float* gy, float* grads);
int fia_debug_precondition(fia_session* s, const float* r, float* z);
/* the grid transfers of the preconditioner: op 0 restriction (fine -> level 0), 1 trilinear
 * prolongation (level 0 -> fine, 0 on excluded cells), 2 adjoint of the prolongation */
int fia_debug_grid_op(fia_session* s, int op, const float* in, float* out);
/* FP32 form: solve B x = rhs (B = -A of the session's Poisson problem; host arrays) with
 * the solver of sp, x starting from 0. */
int fia_debug_solve_rhs(fia_session* s, const float* rhs, float* x, const fia_solver_params* sp,
                        fia_solver_report* rep);
/* capacity of the session's clipped-piece store (either form; it grows when a pass needs more) */
int fia_debug_set_piece_capacity(fia_session* s, long long pieces);
long long fia_debug_piece_capacity(fia_session* s);
/* gradient of the energy-norm loss of pair i with respect to all parameters (no update) */
int fia_debug_learned_grad(fia_session* s, int pair, float* grads, double* loss);
/* the network's tensor-core (tcgen05) convolution path: enable 1 / 0 switches it on / off
 * (on by default; off runs every layer on the mma.sync kernel), -1 leaves it; *status (if
 * not null) receives the path's error bits (bit 0: a bounded wait ran out) */
int fia_debug_learned_tc(fia_session* s, int enable, unsigned* status);
/* FP32 form: the face clipper's shared-memory path: enable 1 / 0 switches it on / off (on
 * by default; off clips every face in local memory, with the same pieces), -1 leaves it;
 * *deferred (if not null) receives the faces the local-memory clipper took since fia_create
 * (faces the shared pool cannot hold, or all faces while the path is off). */
int fia_debug_clip_fast(fia_session* s, int enable, unsigned long long* deferred);
/* FP64 form: enable 1 evaluates every WENO6 interpolation in full, 0 (the default) collapses
 * it along the axes on which the point lies on a node plane of the field (vertices at rest,
 * psi points of the pieces: equal in exact arithmetic, fewer evaluations), -1 leaves it;
 * returns the setting. */
int fia_debug_full_weno(fia_session* s, int enable);
/* FP64 form: enable 1 (the default) runs each pass's faces as the piece pipeline (a thread per
 * face clips and stores its pieces, a thread per piece integrates, a thread per face sums in
 * emission order), 0 as one thread per face that integrates each piece as it is clipped (the
 * same arithmetic and order of sums), -1 leaves it; returns the setting (0 for an FP32C
 * session, which always runs its own piece pipeline). */
int fia_debug_piece_pipeline(fia_session* s, int enable);
/* FP64 form, for sensitivity studies: every backtraced vertex of every later pass is moved by
 * up to `cells` cells (0 <= cells <= 0.5; 0, the default, switches it off) along each axis,
 * independently per vertex, axis and pass (a hash, uniform in [-cells, cells)), before the
 * clamp: perturbations of the size of FP32 rounding of the vertex positions. */
int fia_debug_vertex_jitter(fia_session* s, double cells);

/* Test hooks: single pieces of the path on host data (FP64 buffers), mirroring the oracle. */
/* one flux pass of a node field (comp -1 density, 0..2 velocity) with the session velocity */
int fia_debug_flux_pass(fia_session* s, int comp, const double* field, double dt, int interp, int psi_mode,
                        int use_integral, int zero_velocity, const double* color_off2, int k,
                        double minimal_area, double* out);
/* backtraced vertex positions of the cell lattice of a field (3 doubles per vertex) */
int fia_debug_backtrace(fia_session* s, int comp, double dt, int interp, double* out);
/* psi of a node field (mode 0 plain, 1 WENO6 integral, 2 linear integral) */
int fia_debug_psi(fia_session* s, int comp, const double* field, int mode, int k, double* out);

#ifdef __cplusplus
}
#endif
#endif /* FIA_H */
