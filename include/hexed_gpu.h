/* hexed_gpu.h -- C ABI of the GB300 (sm_103a) DG spatial-operator / stage-update library.
 *
 * The library replaces the OpenMP kernel layer of hexed (ARTLab-GT/hexed): the free
 * functions of include/kernels.hpp:22-42 and the Solver stage loop of
 * src/Solver.cpp:56-133,834-913 that calls them. A caller hands over one flat
 * "mesh arena" (plain host pointers and sizes, described below) that mirrors the
 * storage the reference's Kernel_element / Kernel_connection / Refined_face views
 * point into (include/Kernel_element.hpp:14-45, include/Kernel_connection.hpp:55-102,
 * include/Refined_face.hpp:9-15); the library keeps a device copy and runs every
 * kernel on it. All entry points return 0 on success or a negative hexed_status;
 * hexed_gpu_last_error() gives the message of the last failure in the calling thread.
 *
 * Sizes: nd = n_dim (2 or 3), rs = row_size (2..8), nq = rs^nd, nfq = rs^(nd-1),
 * nv = nd + 2 (momentum[nd], density, total energy; include/pde.hpp:48-50),
 * nvert = 2^nd.
 *
 * Arena layout (all double, C order, outermost index first):
 *   elem      [n_elem][nv + 3][nq]  rows 0..nv-1 conserved state, row nv time-step scale,
 *                                   row nv+1 bulk AV coefficient, row nv+2 Laplacian AV
 *                                   coefficient (src/Element.cpp:119-142, include/pde.hpp:17-21)
 *   rcache    [n_elem][nv][nq]      residual cache (Kernel_element::residual_cache)
 *   face      [n_slot][2][nv][nfq]  face traces; [0] extrapolated state / numerical flux,
 *                                   [1] LDG storage (include/connection.hpp:52-67).
 *                                   Slot e*2nd + i_face is face i_face of element e; slots
 *                                   beyond n_elem*2nd are boundary ghost faces and the fine
 *                                   mortar faces of hanging-node connections.
 *   nom_size  [n_elem]              nominal element edge length
 *   vert_tss  [n_elem][nvert]       vertex time-step scale, already min-shared over vertices
 *   jac       [n_def][nd*nd + 1][nq] reference-level normals [i][j][nq] then Jacobian
 *                                   determinant [nq] (src/Deformed_element.cpp:60-116)
 *   face_nrml [n_def][2nd][nd][nfq] area-weighted face normal each deformed element sees on
 *                                   each face (identity where the reference passes null)
 * Elements are ordered Cartesian first (0..n_car_elem-1), then deformed.
 *
 * Connection lists (int32):
 *   car_con  [n_car_con][3]   slot0, slot1, i_dim  (direction {{d,d},{1,0}}: slot0 is the
 *                             + face of its element, slot1 the - face)
 *   def_con  [n_def_con][3]   slot0, slot1, packed direction:
 *                             i_dim0 | i_dim1 << 2 | face_sign0 << 4 | face_sign1 << 5
 *   def_con_nrml [n_def_con][nd][nfq]  shared face normal in face-0 order (con.normal())
 *   bc_con   [n_bc_con][4]    inside slot, ghost slot, i_dim | inside_face_sign << 2,
 *                             index into bc_spec
 *   bc_nrml  [n_bc_con][nd][nfq]  surface normal of the boundary face (not flipped)
 *   bc_cache [n_bc_con][2][nv][nfq] state cache, flux cache (include/connection.hpp:342-377)
 *   ref_face [n_ref_face][7]  coarse slot, fine mortar slots[4] (-1 = unused), stretch0,
 *                             stretch1 (include/Refined_face.hpp:9-15)
 *   vert_id  [n_elem][nvert]  global vertex index of each element vertex (optional; needed by
 *                             hexed_gpu_set_art_visc_admis, which shares values over vertices)
 */
#ifndef HEXED_GPU_H_
#define HEXED_GPU_H_

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum hexed_status {
  HEXED_OK = 0,
  HEXED_ERR_INVALID = -1,     /* bad argument, e.g. invalid (n_dim, row_size) -- the
                                 reference throws "demand for invalid kernel"
                                 (include/kernel_factory.hpp:111-119) */
  HEXED_ERR_CUDA = -2,        /* CUDA runtime failure */
  HEXED_ERR_NUMERICAL = -3,   /* device kernels flagged a non-finite or non-admissible state */
  HEXED_ERR_NO_DEVICE = -4,   /* no CUDA device visible */
  HEXED_ERR_ALLOC = -5,       /* device memory exhausted */
  HEXED_ERR_PRECONDITION = -6 /* a HEXED_ASSERT of the reference would fire, e.g. two-stage
                                 stabilization requested for diffusion (include/Spatial.hpp:322) */
};

/* Boundary-condition kinds (include/Boundary_condition.hpp, src/Boundary_condition.cpp). */
enum hexed_bc_kind {
  HEXED_BC_FREESTREAM = 0,        /* src/Boundary_condition.cpp:62-76, 299 */
  HEXED_BC_RIEMANN_INVARIANTS = 1,/* src/Boundary_condition.cpp:78-182 */
  HEXED_BC_NONPENETRATION = 2,    /* src/Boundary_condition.cpp:302-344 */
  HEXED_BC_COPY = 3,              /* src/Boundary_condition.cpp:450-458 */
  HEXED_BC_OUTFLOW = 4,           /* src/Boundary_condition.cpp:465-477 */
  HEXED_BC_PRESSURE_OUTFLOW = 5,  /* src/Boundary_condition.cpp:184-223 */
  HEXED_BC_NO_SLIP = 6            /* src/Boundary_condition.cpp:371-427 */
};

/* Thermal sub-model of the no-slip wall (include/Boundary_condition.hpp:140-190). */
enum hexed_thermal_kind {
  HEXED_THERMAL_HEAT_FLUX = 0,    /* Prescribed_heat_flux (default: adiabatic, 0) */
  HEXED_THERMAL_ENERGY = 1,       /* Prescribed_energy (isothermal) */
  HEXED_THERMAL_EQUILIBRIUM = 2   /* Thermal_equilibrium */
};

typedef struct hexed_bc_spec {
  int kind;                /* hexed_bc_kind */
  int thermal_kind;        /* hexed_thermal_kind, no-slip only */
  double freestream[5];    /* conserved freestream state (first nv entries used) */
  double pressure;         /* Pressure_outflow: prescribed pressure */
  double coercion;         /* No_slip heat-flux coercion (reference default 2) */
  double thermal_value;    /* heat flux (HEAT_FLUX) or energy per mass (ENERGY) */
  double emissivity, heat_transfer_coef, temperature; /* Thermal_equilibrium */
} hexed_bc_spec;

/* Transport model: coefficient(sqrt T) = const_val + ref_val (sqrtT/sqrt(ref_temp))^3
 * (ref_temp + temp_offset)/(T + temp_offset) (include/Transport_model.hpp:21-44). */
typedef struct hexed_transport {
  double const_val, ref_val, ref_temp, temp_offset;
  int is_viscous;
} hexed_transport;

typedef struct hexed_mesh_desc {
  int n_dim, row_size;
  int n_car_elem, n_def_elem;
  int n_slot;
  int n_car_con, n_def_con, n_bc_con, n_ref_face, n_bc_spec;
  double* elem;
  double* rcache;
  double* face;
  const double* nom_size;
  const double* vert_tss;
  const double* jac;
  const double* face_nrml;
  const int* car_con;
  const int* def_con;
  const double* def_con_nrml;
  const int* bc_con;
  const double* bc_nrml;
  double* bc_cache;
  const int* ref_face;
  const hexed_bc_spec* bc_spec;
  int n_vert;              /* number of distinct vertices (0: no vertex table) */
  const int* vert_id;
} hexed_mesh_desc;

/* Arrays that can be copied in and out of the device arena. */
enum hexed_array {
  HEXED_ARRAY_ELEM = 0,
  HEXED_ARRAY_RCACHE = 1,
  HEXED_ARRAY_FACE = 2,
  HEXED_ARRAY_BC_CACHE = 3,
  HEXED_ARRAY_NOM_SIZE = 4,
  HEXED_ARRAY_VERT_TSS = 5,
  HEXED_ARRAY_BC_NRML = 6,
  HEXED_ARRAY_REF_STATE = 7,  /* mixed form only: [n_elem][nv] reference state of each element
                                 (write it before the element's state and traces) */
  HEXED_ARRAY_JAC = 8,        /* [n_def][nd*nd + 1][nq] (read / write) */
  HEXED_ARRAY_FACE_NRML = 9,  /* [n_def][2nd][nd][nfq] */
  HEXED_ARRAY_DEF_CON_NRML = 10, /* [n_def_con][nd][nfq] */
  HEXED_ARRAY_SAV_AUX = 11,   /* smoothness-based AV storage [n_elem][4 + 2 rs][nq]: the four
                                 forcing rows, the advection state (rs rows, 1 at creation) and
                                 its residual cache (rs rows); allocated on first use */
  HEXED_ARRAY_SAV_FACE = 12   /* smoothness-based AV face slots [n_slot][max(2 nv, nd + rs) nfq]
                                 (the size of a reference Face_connection face), LDG half at
                                 nv nfq; allocated on first use */
};

/* Arithmetic of the volume and face kernels. */
enum hexed_precision {
  HEXED_FP64 = 0,   /* everything in double: the parity path */
  HEXED_MIXED = 1   /* fluxes, derivatives and face traces in float; state, stage update,
                       metrics, time step and residual norms in double */
};

/* Parameters of one Solver::update (src/Solver.cpp:834-886, defaults set at 151-174). */
typedef struct hexed_update_params {
  double max_safety;     /* "max_safety" (CFL fraction of the basis limit) */
  double max_time_step;  /* "max_time_step" */
  int n_cheby_flow;      /* Chebyshev sub-steps */
  int flow_iters;        /* repetitions per update */
  int local_time;        /* local time stepping */
  int use_filter;        /* modal filter */
  int use_ldg;           /* viscous / artificial-viscosity path (Solver::use_ldg) */
  hexed_transport visc, cond;
  double av_admis_char_speed; /* > 0: Solver::set_art_visc_admis with this characteristic
                                 speed before every update, as Case.cpp:432 does when
                                 "diffusive_admissibility" is set; 0: off */
  int fix_admis;              /* Solver::set_fix_admissibility (src/Solver.cpp:667-670): after
                                 each stage, Solver::fix_admissibility restores thermodynamic
                                 admissibility (on with set_shock, include/Case.hil:95) */
  double fix_admis_max_safety; /* "fix_admis_max_safety" (src/Solver.cpp:153; default 0.7) */
} hexed_update_params;

typedef struct hexed_gpu_ctx hexed_gpu_ctx;

/* Thread-local message of the last failing call. */
const char* hexed_gpu_last_error(void);

/* Library build information: "sm_103a" plus the maximum row size. */
const char* hexed_gpu_version(void);

/* Creates a context on the current CUDA device and uploads the whole arena.
 * Replaces the setup the reference performs once per mesh (Solver::calc_jacobian +
 * initialize, src/Solver.cpp:273-408) as far as the kernels see it. `elem`, `rcache`,
 * `face` and `bc_cache` may be null: their device copies then start at zero (an arena whose
 * states are written later with hexed_gpu_write_range). */
int hexed_gpu_create(const hexed_mesh_desc* desc, int precision, hexed_gpu_ctx** out);
int hexed_gpu_destroy(hexed_gpu_ctx* ctx);

/* Host <-> device copies of one arena array (hexed_array); sizes follow the layout above. */
int hexed_gpu_upload(hexed_gpu_ctx* ctx, int which, const double* host);
int hexed_gpu_download(hexed_gpu_ctx* ctx, int which, double* host);
int hexed_gpu_synchronize(hexed_gpu_ctx* ctx);

/* --- kernel layer: one call per free function of include/kernels.hpp:22-42 --- */

/* compute_euler (src/kernels_convective.cpp:8-19, 36): Neighbor (Cartesian, deformed and
 * boundary connections), Restrict_refined, Local, Prolong_refined. */
int hexed_gpu_compute_euler(hexed_gpu_ctx* ctx, double dt, int i_stage, int compute_residual,
                            int use_filter);

/* compute_navier_stokes (src/kernels_diffusive.cpp:8-32): the LDG chain. The flux
 * boundary conditions (Solver::apply_flux_bcs, src/Solver.cpp:69-81) run on the device
 * between Prolong and Neighbor_reconcile, so no host callback is needed. */
int hexed_gpu_compute_navier_stokes(hexed_gpu_ctx* ctx, double dt, int i_stage,
                                    int compute_residual, int use_filter,
                                    const hexed_transport* visc, const hexed_transport* cond);

/* max_dt_euler / max_dt_navier_stokes (src/kernels_max_dt.cpp:8-21): writes the local
 * time-step scale (local_time) or returns the global step in *out_dt. */
int hexed_gpu_max_dt(hexed_gpu_ctx* ctx, double convective_safety, double diffusive_safety,
                     int local_time, int use_filter, int viscous, const hexed_transport* visc,
                     const hexed_transport* cond, double* out_dt);

/* compute_prolong / compute_restrict / compute_write_face (src/kernels_convective.cpp:21-44). */
int hexed_gpu_compute_prolong(hexed_gpu_ctx* ctx, int scale, int offset);
int hexed_gpu_compute_restrict(hexed_gpu_ctx* ctx, int scale, int offset);
int hexed_gpu_compute_write_face(hexed_gpu_ctx* ctx);

/* Metric set-up on the device: Deformed_element::set_jacobian (src/Deformed_element.cpp:15-134)
 * for every deformed element from its vertex positions vert_pos [n_def][nvert][nd] (vertex bit
 * d <-> reference dimension d, dim 0 most significant), then the connection part of
 * Solver::calc_jacobian (src/Solver.cpp:273-381): shared normals of the deformed connections,
 * boundary normals, and the vertex time-step scale shared (minimum) over the vertex table when
 * the arena has one. Overwrites jac, face_nrml, def_con_nrml, bc_nrml and vert_tss of the
 * arena. For conforming deformed meshes (hanging faces only between Cartesian elements, as
 * the arena builds them). */
int hexed_gpu_compute_jacobian(hexed_gpu_ctx* ctx, const double* vert_pos);

/* Solver::is_admissible (src/Solver.cpp:921-959, thermo::admissible src/thermo.cpp:6-18):
 * *admissible = 1 if density and total energy are positive at every point of every element
 * state, element face trace and fine mortar face, else 0. record (optional, [n_elem] of the
 * active elements) receives 1 for each inadmissible element. Returns HEXED_ERR_NUMERICAL
 * ("state is not finite") if any of these values is not finite, where the reference asserts. */
int hexed_gpu_is_admissible(hexed_gpu_ctx* ctx, int* admissible, int* record);

/* Solver::fix_admissibility (src/Solver.cpp:961-1095). While the state is not admissible
 * (hexed_gpu_is_admissible), and then for as many iterations again as it took, diffuse the
 * state with pde::Fix_therm_admis (include/pde.hpp:437-493): local time step at
 * `stability_ratio`, two sub-steps of the LDG diffusion chain with ghost state = inside and
 * ghost LDG flux = -inside at the boundaries, then the flow's Max_dt of p (its step is
 * kept). *iterations: the count the reference returns (0: was admissible). Fails with
 * HEXED_ERR_NUMERICAL for a non-finite state or after 100000 iterations, as the reference
 * asserts. Synchronizes the stream on every iteration. */
int hexed_gpu_fix_admissibility(hexed_gpu_ctx* ctx, const hexed_update_params* p, double stability_ratio,
                                int* iterations);

/* Flags the kernels raised since the context was created (0 = none). Bit 0: a volume kernel
 * gave up waiting for the bulk copy of its element states and read global memory instead
 * (results are unaffected; the copy is slower than it should be). No counterpart in the
 * reference. */
int hexed_gpu_device_flags(hexed_gpu_ctx* ctx, int* flags);

/* Checks the double <-> float conversions the mixed form does with integer operations against
 * the hardware conversions on n host values; *mismatches = values whose results differ in
 * any bit (values whose float result is subnormal are skipped: the mixed form flushes them
 * to zero). A diagnostic; no counterpart in the reference. */
int hexed_gpu_check_conversions(const double* values, long n, long* mismatches);

/* Launch shape of the volume and face kernels. local_variant selects the elements per CTA of
 * the 2D Cartesian volume kernels: 0 = 256/nq (the default), 1 = half, 2 = twice that (3D
 * kernels have only 0). face_threads (64, 128 or 256 = default) is the CTA size of the
 * face kernels. Chosen per row size by the autotuner of the serving loop; results do not
 * depend on it. No counterpart in the reference. */
int hexed_gpu_set_launch_shape(hexed_gpu_ctx* ctx, int local_variant, int face_threads);
/* The launch shape in use: elements per volume-kernel CTA and face-kernel threads per CTA. */
int hexed_gpu_launch_shape(hexed_gpu_ctx* ctx, int* local_elems_per_cta, int* face_threads);

/* Reference state (nv conserved values) of every element in the mixed form. The mixed form
 * stores face traces, and forms convective fluxes, as differences from the element's
 * reference state, so that float arithmetic resolves small variations of the flow. By default
 * each element's reference is the mean of its own state given to hexed_gpu_create, so the
 * float offsets carry only the variation inside the element; neighbouring elements with
 * different references exchange traces and fluxes through the exact difference of their
 * references. This call gives every element the same state; HEXED_ARRAY_REF_STATE sets it
 * per element. Call this before the states and traces it applies to are written. No effect
 * in the FP64 form. No counterpart in the reference. */
int hexed_gpu_set_reference_state(hexed_gpu_ctx* ctx, const double* state);

/* The conserved state of the active elements as host arrays [n_elem][nv][nq] (the first nv
 * rows of each element of the arena, without the time-step and AV rows): the copy a caller
 * whose state lives in host memory makes around each update, as the reference's elements hold
 * it (Element::state(), src/Element.cpp:119-142). Returns when the copy is complete. Pinned
 * host memory gives the full transfer rate. write_state stages the host array in device
 * memory (n_elem nv nq doubles, allocated on the first call) and scatters it into the
 * arena; read_state is one strided copy. */
int hexed_gpu_write_state(hexed_gpu_ctx* ctx, const double* state);
int hexed_gpu_read_state(hexed_gpu_ctx* ctx, double* state);

/* Write_face for elements [elem_begin, elem_begin + elem_count) only: initialises the face
 * traces of one newly admitted solve without touching the traces of solves already running.
 * No counterpart in the reference (which writes the faces of a whole mesh at once). */
int hexed_gpu_write_face_range(hexed_gpu_ctx* ctx, int elem_begin, int elem_count);

/* Solver::set_art_visc_admis (src/Solver.cpp:636-658): per-element smoothness indicator of
 * the specific volume (Stab_art_visc, src/stabilizing_art_visc.cpp:8-66) scaled by
 * char_speed, maximum over the elements sharing each vertex, multilinear interpolation to
 * the quadrature points into the Laplacian AV row. Needs the arena's vertex table. */
int hexed_gpu_set_art_visc_admis(hexed_gpu_ctx* ctx, double char_speed);

/* Settings of Solver::update_art_visc_smoothness (src/Solver.cpp:457-582) and
 * Solver::diffuse_art_visc (src/Solver.cpp:428-455); the reference's defaults
 * (src/Solver.cpp:154-163) in brackets. */
typedef struct hexed_sav_params {
  double advect_length;      /* the `advect_length` argument (Case: art_visc_width) */
  int advect_iters;          /* av_advect_iters [1] */
  int diff_iters;            /* av_diff_iters [1] */
  int n_cheby;               /* n_cheby_av [1] */
  int av_row_size;           /* av_rs, degree + 1 of the projected Legendre mode [row_size] */
  double advect_safety;      /* av_advect_max_safety [0.7] */
  double diff_safety;        /* av_diff_max_safety [0.7] */
  double diff_ratio;         /* av_diff_ratio [0.3] */
  double visc_mult;          /* av_visc_mult [100] */
  double unscaled_max;       /* av_unscaled_max [5] */
  double freestream_mass;    /* freestream{n_dim} */
  double freestream_energy;  /* freestream{n_dim + 1} */
} hexed_sav_params;

/* Solver::update_art_visc_smoothness (src/Solver.cpp:457-582): the smoothness-based artificial
 * viscosity of set_shock. advect_iters pseudo-time iterations of pde::Advection (two stages,
 * local time step) estimate a high-order derivative of the flow; its projection onto the
 * Legendre mode of degree av_row_size - 1 is smeared by n_forcing - 1 = 3 implicit diffusion
 * steps of pde::Smooth_art_visc (diff_iters x n_cheby sub-steps, Solver::diffuse_art_visc);
 * the bulk AV row receives us_max f/(us_max + f). The flow state is restored and its face
 * traces re-extrapolated (Write_face, Prolong); the time-step-scale row holds the last
 * pseudo-time step, as in the reference. *residual (may be NULL) receives art_visc_residual
 * (reading it synchronizes). The storage of HEXED_ARRAY_SAV_AUX / HEXED_ARRAY_SAV_FACE is
 * allocated on the first call and persists: the advection state carries over between calls
 * as the reference's element storage does. FP64 arithmetic in both precision forms. */
int hexed_gpu_update_art_visc_smoothness(hexed_gpu_ctx* ctx, const hexed_sav_params* params, double* residual);

/* Solver::apply_state_bcs / apply_flux_bcs (src/Solver.cpp:56-81). */
int hexed_gpu_apply_state_bcs(hexed_gpu_ctx* ctx);
int hexed_gpu_apply_flux_bcs(hexed_gpu_ctx* ctx);

/* --- solver layer --- */

/* Solver::update (src/Solver.cpp:834-886): time step, state BCs and both stages, all
 * enqueued without a host round trip (the time step stays on the device). *out_dt
 * (may be NULL) receives the last step taken; reading it synchronizes. */
int hexed_gpu_update(hexed_gpu_ctx* ctx, const hexed_update_params* params, double* out_dt);

/* Solver::compute_residual (src/Solver.cpp:899-913). */
int hexed_gpu_compute_residual(hexed_gpu_ctx* ctx, const hexed_update_params* params);

/* Residual norms of Case.hil's compute_residuals (src/Solver.cpp:1113-1131,
 * src/Qpoint_func.cpp:37-45): sqrt of the integral of (rcache/tss)^2 over the domain,
 * summed over momentum components, density, energy -> out[3]. */
int hexed_gpu_residual_norm(hexed_gpu_ctx* ctx, double out[3]);

/* --- continuous batching: many independent solves in one arena ---
 * A serving loop packs the meshes of many independent solves into one Cartesian arena of
 * fixed capacity (connections never cross solves), lets the kernels run over an active
 * prefix, and admits / retires solves by rewriting ranges of the arena. Per-solve residual
 * norms are segmented reductions over each solve's element range, so a solve's arithmetic is
 * the same alone and in the mix. No counterpart in the reference, which runs one solve per
 * process. */

/* Host <-> device copy of `count` entries of an arena array starting at entry `offset`
 * (entries in units of the array's scalar type). `which` is a hexed_array. */
int hexed_gpu_write_range(hexed_gpu_ctx* ctx, int which, long offset, long count, const double* host);
int hexed_gpu_read_range(hexed_gpu_ctx* ctx, int which, long offset, long count, double* host);

/* Int connection arrays for hexed_gpu_write_int_range. */
enum hexed_int_array {
  HEXED_INT_CAR_CON = 0,   /* [n][3] */
  HEXED_INT_BC_CON = 1     /* [n][4] */
};
/* Rewrites rows of a connection array; every entry is range-checked against the arena
 * (slots, dimensions, boundary-condition index) before it reaches the device. offset and
 * count are in rows. */
int hexed_gpu_write_int_range(hexed_gpu_ctx* ctx, int which, long offset, long count, const int* host);

/* Replaces boundary-condition record `index` (< n_bc_spec of the arena). */
int hexed_gpu_write_bc_spec(hexed_gpu_ctx* ctx, int index, const hexed_bc_spec* spec);

/* Active prefix the kernels process in a Cartesian-only arena: elements [0, n_car_elem),
 * Cartesian connections [0, n_car_con), boundary connections [0, n_bc_con); each at most the
 * arena's size. */
int hexed_gpu_set_active(hexed_gpu_ctx* ctx, int n_car_elem, int n_car_con, int n_bc_con);

/* Residual norms (as hexed_gpu_residual_norm) of each of n_seg element segments
 * [elem_begin[i], elem_begin[i] + elem_count[i]): out[3*i .. 3*i+2]. One CTA reduces one
 * segment in a fixed order, so a segment's norms do not depend on the other segments. */
int hexed_gpu_segment_residual_norms(hexed_gpu_ctx* ctx, int n_seg, const int* elem_begin,
                                     const int* elem_count, double* out);

/* Largest n_seg hexed_gpu_segment_residual_norms_static accepts. */
#define HEXED_STATIC_MAX_SEGMENTS 4096

/* hexed_gpu_segment_residual_norms without any device allocation: same arguments, same
 * results. hexed_gpu_segment_residual_norms grows its per-context table and output buffers
 * with cudaMalloc when n_seg exceeds what it has seen; this variant instead uses one
 * fixed array of module memory (128 KiB per device, up to HEXED_STATIC_MAX_SEGMENTS
 * segments; more are rejected with HEXED_ERR_INVALID). It is for callers that cannot let
 * the library allocate: a serving loop that has handed out the device's free memory to
 * admitted solves, or one that keeps a fixed memory budget, would otherwise see a failed or
 * device-synchronising allocation in the middle of its loop. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress); make that first call before
 * any stream capture. The array is shared by every context on the device and keeps the last
 * call's contents, so overlapping calls (from two threads, or on two streams) race: callers
 * serialise them. No counterpart in the reference. */
int hexed_gpu_segment_residual_norms_static(hexed_gpu_ctx* ctx, int n_seg, const int* elem_begin,
                                            const int* elem_count, double* out);

/* n consecutive Solver::update steps. use_graph != 0 captures the n-step launch sequence into
 * a CUDA graph on first use and replays it while the parameters and active sizes are
 * unchanged (launch overhead of small solves). */
int hexed_gpu_update_n(hexed_gpu_ctx* ctx, const hexed_update_params* params, int n, int use_graph);

/* --- instrumentation --- */

/* Per-kernel CUDA-event timing on the context's stream, the device counterpart of the
 * reference's per-kernel stopwatch hooks (include/kernel_factory.hpp:32-45,
 * src/Stopwatch_tree.cpp). enable != 0 starts recording (and clears earlier records). */
int hexed_gpu_profile_enable(hexed_gpu_ctx* ctx, int enable);

typedef struct hexed_kernel_time {
  char name[48];
  int launches;
  double total_ms;
} hexed_kernel_time;

/* Waits for the recorded launches and reports launches and total device time per kernel
 * (at most `capacity` entries; *n_out = number written). Clears the records. */
int hexed_gpu_profile_read(hexed_gpu_ctx* ctx, hexed_kernel_time* out, int capacity, int* n_out);

/* The cudaStream_t every kernel of the context runs on (for callers that time or order
 * work against it). No counterpart in the reference, which has no device stream. */
void* hexed_gpu_stream(hexed_gpu_ctx* ctx);

/* Measures the FP64 FMA throughput of the current device with a dependent-chain DFMA
 * kernel (TFLOP/s, 2 flops per FMA) -- the FP64 roofline denominator. No counterpart in
 * the reference. */
int hexed_gpu_fp64_peak(double* tflops);

#ifdef __cplusplus
}
#endif
#endif
