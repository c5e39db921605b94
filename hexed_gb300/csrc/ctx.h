// ctx.h -- device context behind the opaque hexed_gpu_ctx handle.
#pragma once
#include <cuda_runtime.h>
#include "../../include/hexed_gpu.h"

namespace hx {

struct HostTables {
  const double* node; const double* weight; const double* diff; const double* bound;
  const double* filter; const double* prolong; const double* restrict_; const double* ortho;
  double max_cfl, min_eig_diffusion, step_ratio;
};

struct Ctx;
struct LocalDt;   // kernels.cuh

// Per-kernel CUDA-event timing, the device analogue of the reference's per-kernel
// Stopwatch_tree hooks (include/kernel_factory.hpp:32-45). Off unless enabled.
struct Profiler {
  static constexpr int max_events = 8192;
  static constexpr int max_names = 64;
  bool enabled = false;
  cudaEvent_t events[max_events];
  int event_name[max_events/2];
  int n_pairs = 0;
  bool created = false;
  const char* names[max_names];
  int n_names = 0;
  int launches[max_names];
  double total_ms[max_names];
};

// Launch sequences of one (n_dim, row_size, precision); all enqueue on Ctx::stream.
struct OpsTable {
  void (*compute_euler)(Ctx&, int stage, int compute_residual, int use_filter, bool fuse_bc, const LocalDt& ldt);
  void (*compute_navier_stokes)(Ctx&, int stage, int compute_residual, int use_filter,
                                const hexed_transport& visc, const hexed_transport& cond, bool fuse_bc);
  void (*max_dt)(Ctx&, double msc, double msd, int local_time, int viscous, const hexed_transport& visc,
                 const hexed_transport& cond, double max_time_step, double cheby);
  void (*refine)(Ctx&, bool prolong, bool scale, bool offset);
  void (*write_face)(Ctx&, int e_begin, int n_elem);
  void (*bc_state)(Ctx&);
  void (*bc_flux)(Ctx&);
  void (*residual_norm)(Ctx&, double* d_out);
  void (*set_art_visc_admis)(Ctx&, double char_speed);
  void (*segment_residual_norms)(Ctx&, int n_seg, const int* d_begin, const int* d_count, double* d_out);
  int (*local_elems_per_cta)(int variant);
  void (*admissible)(Ctx&, int* d_record);
  void (*compute_jacobian)(Ctx&, const double* d_vert_pos, double* d_fn, double* d_vtss);
  void (*fix_admis_coef)(Ctx&, const int* d_record, bool swap_only);
  void (*ref_terms)(Ctx&);
  void (*update_art_visc_smoothness)(Ctx&, const hexed_sav_params&, double* d_residual);
  int (*sav_slot_dof)();
};

// A captured multi-update sequence and the inputs it was captured for.
struct GraphCache {
  bool valid = false;
  cudaGraphExec_t exec = nullptr;
  hexed_update_params params;
  int n = 0, n_car = 0, n_car_con = 0, n_bc_con = 0;
};

struct Ctx {
  int nd, rs, precision, device;
  int n_car, n_def, n_slot, n_car_con, n_def_con, n_bc_con, n_ref, n_bc_spec;
  size_t nq, nfq, nv;
  cudaStream_t stream;
  HostTables tables;
  const OpsTable* ops;
  // device arena
  double* elem; double* rcache; double* face;
  double* nom_size; double* vert_tss; double* jac; double* face_nrml;
  int* car_con; int* def_con; double* def_con_nrml;
  int* bc_con; double* bc_nrml; double* bc_cache; int* ref_face; hexed_bc_spec* bc_spec;
  int n_vert; int* vert_id;            // vertex table (optional)
  double* uncert; double* vmax;        // artificial-viscosity scratch: [n_elem], [n_vert]
  // scratch
  double* scalars;       // SC_* slots
  double* partials;      // reduction partials, max_partials doubles
  int max_partials;
  int* status;
  unsigned* dt_ticket;   // CTAs of k_max_dt done; the last one takes the minimum and resets it
  double* d_norm;        // residual norm output [3]
  double* h_pinned;      // pinned host staging for scalars [8]
  Profiler* prof;
  // sizes of the arena arrays (the n_* counts above are the active prefix the kernels see)
  int cap_car, cap_car_con, cap_bc_con;
  // per-call scratch of the segmented residual norms
  int seg_capacity;
  int* seg_table;        // device [2][seg_capacity]
  double* seg_out;       // device [3*seg_capacity]
  GraphCache* graph;
  bool capturing;
  // Jacobian determinant reciprocal [n_def][nq] (both forms)
  double* inv_det;
  // contiguous staging of hexed_gpu_write_state [n_elem][nv][nq] (allocated on first use)
  double* state_stage;
  // mixed form: FP32 face traces, residual cache and metric-normal copies, and the reference
  // state of each element [n_elem][nv] the traces and fluxes are offsets from (by default the
  // mean conserved state of the initial state)
  float* face_f; float* rcache_f; float* nrm_f; float* face_nrml_f; float* def_con_nrml_f; float* bc_nrml_f;
  float* vert_tss_f;     // FP32 vertex time-step scales [n_elem][2^nd] (Max_dt)
  double* ref_state;
  // its terms in float for the offset fluxes (RefState: state and its rounding error, velocity,
  // |v|^2, enthalpy, 1/density), [n_elem][3 nd + 7], refreshed whenever ref_state changes
  float* ref_terms;
  // element of each slot beyond the element slots (ghost: the inside element; hanging-face
  // mortar: the coarse element), whose reference state the slot's traces are offsets from
  int* slot_elem;
  int* record;           // per-element admissibility records [cap elements] (allocated at creation)
  // launch shape: volume-kernel variant (elements per CTA, see Runner::epb_of) and threads
  // per CTA of the face kernels
  int local_variant;
  int face_threads;
  // 1 while Solver::fix_admissibility's diffusion runs: the kernels compute pde::Fix_therm_admis
  int fta;
  // smoothness-based AV storage (allocated on first use): [cap elements][4 + 2 rs][nq],
  // [n_slot][sav slot_dof], and per-element residual partials [cap elements]
  double* sav_aux; double* sav_face; double* sav_partials;
};

// Max_dt's CFL reciprocals for convective and diffusive safety factors (include/Spatial.hpp:
// 776-777): uniform over a launch, so formed once on the host
inline double inv_cfl_conv(const Ctx& c, double msc) { return 1./(c.tables.max_cfl*msc); }
inline double inv_cfl_diff(const Ctx& c, double msd) { return 1./(-2/c.tables.min_eig_diffusion*msd); }

// Bracket one launch with timing events when profiling is enabled.
struct ProfScope {
  Ctx& c; int pair;
  ProfScope(Ctx& ctx, const char* name);
  ~ProfScope();
};

const OpsTable* ops_2_2(int); const OpsTable* ops_2_3(int); const OpsTable* ops_2_4(int);
const OpsTable* ops_2_5(int); const OpsTable* ops_2_6(int); const OpsTable* ops_2_7(int);
const OpsTable* ops_2_8(int);
const OpsTable* ops_3_2(int); const OpsTable* ops_3_3(int); const OpsTable* ops_3_4(int);
const OpsTable* ops_3_5(int); const OpsTable* ops_3_6(int); const OpsTable* ops_3_7(int);
const OpsTable* ops_3_8(int);

} // namespace hx
