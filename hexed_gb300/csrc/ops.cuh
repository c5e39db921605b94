// ops.cuh -- host-side launch sequences for one (n_dim, row_size).
//
// The instantiation units (inst_<nd>_<rs>.cu) include this file once each, so the
// kernels of different row sizes compile in parallel. The sequences mirror the
// reference's kernel calls: compute_euler (src/kernels_convective.cpp:8-19),
// compute_navier_stokes (src/kernels_diffusive.cpp:8-32), max_dt_* (src/kernels_max_dt.cpp).
#pragma once
#include "kernels.cuh"
#include "metrics.cuh"
#include "sav.cuh"
#include "ctx.h"

namespace hx {

inline int grid_for(long items, int block, int max_blocks = 152*16)
{
  long g = (items + block - 1)/block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return int(g);
}

template <int ND, int RS, typename R>
struct Runner
{
  using S = Shape<ND, RS>;
  using FaceT = R;   // storage of traces, residual cache and metric normals (see Dev)

  static Dev<FaceT> dev(Ctx& c)
  {
    Dev<FaceT> m;
    m.n_car = c.n_car; m.n_def = c.n_def; m.n_elem = c.n_car + c.n_def; m.n_slot = c.n_slot;
    m.n_car_con = c.n_car_con; m.n_def_con = c.n_def_con; m.n_bc_con = c.n_bc_con; m.n_ref = c.n_ref;
    m.elem = c.elem;
    m.nom_size = c.nom_size; m.vert_tss = c.vert_tss; m.vert_tss_f = c.vert_tss_f; m.jac = c.jac;
    m.inv_det = c.inv_det;
    m.car_con = c.car_con; m.def_con = c.def_con;
    m.bc_con = c.bc_con; m.bc_nrml = c.bc_nrml; m.bc_cache = c.bc_cache; m.ref_face = c.ref_face;
    m.bc_spec = c.bc_spec; m.scalars = c.scalars; m.partials = c.partials; m.status = c.status;
    m.fta = c.fta;
    if constexpr (std::is_same<R, double>::value) {
      m.rcache = c.rcache; m.face = c.face; m.nrm = c.jac; m.face_nrml = c.face_nrml;
      m.def_con_nrml = c.def_con_nrml; m.bc_nrml_t = c.bc_nrml;
      m.ref = nullptr;
      m.ref_terms = nullptr;
      m.elem_slot_end = 0;
      m.slot_elem = nullptr;
    } else {
      m.rcache = c.rcache_f; m.face = c.face_f; m.nrm = c.nrm_f; m.face_nrml = c.face_nrml_f;
      m.def_con_nrml = c.def_con_nrml_f; m.bc_nrml_t = c.bc_nrml_f;
      m.ref = c.ref_state;
      m.ref_terms = c.ref_terms;
      m.elem_slot_end = (c.cap_car + c.n_def)*2*ND;
      m.slot_elem = c.slot_elem;
    }
    return m;
  }

  static Tab<RS> tab(const Ctx& c)
  {
    Tab<RS> t;
    const HostTables& h = c.tables;
    for (int i = 0; i < RS*RS; ++i) { t.diff[i] = h.diff[i]; t.filter[i] = h.filter[i]; }
    for (int i = 0; i < 2*RS; ++i) { t.bound[i] = h.bound[i]; }
    for (int i = 0; i < RS; ++i) {
      double inv_w = 1./h.weight[i];
      t.lift[i*2] = -(inv_w*h.bound[i]);
      t.lift[i*2 + 1] = inv_w*h.bound[RS + i];
      t.node[i] = h.node[i];
      t.weight[i] = h.weight[i];
    }
    for (int i = 0; i < 2*RS*RS; ++i) { t.prolong[i] = h.prolong[i]; t.restrict_[i] = h.restrict_[i]; }
    for (int i = 0; i < RS; ++i) t.ortho_last[i] = h.ortho[(RS - 1)*RS + i];
    t.max_cfl = h.max_cfl; t.min_eig_diffusion = h.min_eig_diffusion; t.step_ratio = h.step_ratio;
    return t;
  }

  static AvRamp av_ramp()
  {
    AvRamp r;
    r.center = -4.25*std::log(double(RS - 1))/std::log(10.);
    r.half_width = 0.5;
    r.lo = std::pow(10., r.center - r.half_width);
    r.hi = std::pow(10., r.center + r.half_width);
    return r;
  }

  static AvTab<RS, R> av_tab(const Ctx& c)
  {
    const Tab<RS> t = tab(c);
    AvTab<RS, R> a;
    for (int i = 0; i < RS; ++i) {
      a.w[i] = R(t.weight[i]);
      a.ow[i] = R(t.ortho_last[i]*t.weight[i]);
      a.node[i] = R(t.node[i]);
    }
    return a;
  }

  // Elements per CTA of the volume kernel for launch-shape variant v: 0 the default
  // (256/nq), 1 half of it, 2 twice it. The 2D Cartesian kernels (the serving path) are
  // compiled in all three shapes; other kernels only in the default.
  static constexpr int epb_of(int v) { return v == 1 ? (S::epb > 1 ? S::epb/2 : 1) : v == 2 ? 2*S::epb : S::epb; }
  static constexpr bool has_variants(bool def) { return ND == 2 && !def; }

  template <bool DEF, bool VISC, int EPB>
  static void local_shape(Ctx& c, int stage, int cr, int uf, const hexed_transport& visc, const hexed_transport& cond,
                          int e_begin, int e_end, const LocalDt& ldt)
  {
    const int blocks = (e_end - e_begin + EPB - 1)/EPB;
    constexpr size_t smem = LocalSmem<ND, RS, R, DEF, VISC, EPB>::bytes;
    // 3D kernels of row size >= 6 are register-capped for more resident CTAs: 72 registers
    // per thread for the float viscous kernel and 56 for the float inviscid one (4 and 5 CTAs
    // per SM at row size 6, where shared memory allows as many), 128 for the FP64 viscous
    // kernel (2). Below row size 6 the float inviscid kernel is held at 64 (4 CTAs of 256
    // threads): at 66 registers the row-size-4 kernel lost a CTA per SM and ran 19% slower.
    constexpr bool f32 = std::is_same<R, float>::value;
    constexpr int threads = Tile<ND, RS, EPB>::threads;
    constexpr int cap = f32 ? (VISC ? 72 : S::nq > 128 ? 56 : 64) : VISC ? 128 : 0;
    constexpr bool capped = ND == 3 && (S::nq > 128 || (f32 && !VISC));
    constexpr int minb = (cap && capped && 65536/(threads*cap) > 1) ? 65536/(threads*cap) : 1;
    auto kern = k_local<ND, RS, R, DEF, VISC, FaceT, EPB, minb>;
    static bool configured = false;
    if (!configured) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      configured = true;
    }
    ProfScope ps(c, DEF ? (VISC ? "local_def_ns" : "local_def_euler") : (VISC ? "local_car_ns" : "local_car_euler"));
    const Tab<RS> t = tab(c);
    kern<<<blocks, threads, smem, c.stream>>>(dev(c), t, make_rowtab<RS, R>(t), e_begin, e_end, stage, cr, uf,
                                              make_tm<R>(visc), make_tm<R>(cond), ldt);
  }

  template <bool DEF, bool VISC>
  static void local(Ctx& c, int stage, int cr, int uf, const hexed_transport& visc, const hexed_transport& cond,
                    const LocalDt& ldt = LocalDt{0, 0., 0., 0.})
  {
    const int e_begin = DEF ? c.n_car : 0;
    const int e_end = DEF ? c.n_car + c.n_def : c.n_car;
    if (e_end <= e_begin) return;
    if constexpr (has_variants(DEF)) {
      if (c.local_variant == 1)
        return local_shape<DEF, VISC, epb_of(1)>(c, stage, cr, uf, visc, cond, e_begin, e_end, ldt);
      if (c.local_variant == 2)
        return local_shape<DEF, VISC, epb_of(2)>(c, stage, cr, uf, visc, cond, e_begin, e_end, ldt);
    }
    local_shape<DEF, VISC, S::epb>(c, stage, cr, uf, visc, cond, e_begin, e_end, ldt);
  }

  static int local_elems_per_cta(int v) { return has_variants(false) ? epb_of(v) : S::epb; }

  // Deformed_element::set_jacobian + Solver::calc_jacobian (metrics.cuh) from the deformed
  // elements' vertex positions d_vert_pos [n_def][nvert][nd]; d_fn [n_def][2nd][nd][nfq] and
  // d_vtss [n_def][nvert] are scratch. Leaves jac, face_nrml, def_con_nrml, bc_nrml, vert_tss.
  static void compute_jacobian(Ctx& c, const double* d_vert_pos, double* d_fn, double* d_vtss)
  {
    if (c.n_def) {
      constexpr size_t smem = MetricSmem<ND, RS>::bytes;
      static bool configured = false;
      if (!configured) {
        cudaFuncSetAttribute(k_set_jacobian<ND, RS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
      }
      ProfScope ps(c, "set_jacobian");
      k_set_jacobian<ND, RS><<<c.n_def, (S::nq + 31)/32*32, smem, c.stream>>>(d_vert_pos, c.nom_size + c.n_car, tab(c),
                                                                             c.jac, d_fn, d_vtss);
      k_identity_face_normals<ND, RS><<<grid_for((long)c.n_def*2*ND*ND*S::nfq, 256), 256, 0, c.stream>>>(c.face_nrml,
                                                                                                      c.n_def);
      if (c.n_def_con)
        k_def_con_normals<ND, RS><<<grid_for((long)c.n_def_con*S::nfq, 256), 256, 0, c.stream>>>(
            c.def_con, c.n_def_con, c.n_car, d_fn, c.face_nrml, c.def_con_nrml);
    }
    if (c.n_bc_con)
      k_bc_normals<ND, RS><<<grid_for((long)c.n_bc_con*S::nfq, 256), 256, 0, c.stream>>>(c.bc_con, c.n_bc_con, c.n_car,
                                                                                      d_fn, c.face_nrml, c.bc_nrml);
    const int n_elem = c.n_car + c.n_def;
    k_element_vtss<ND><<<grid_for((long)n_elem*S::nvert, 256), 256, 0, c.stream>>>(c.nom_size, c.n_car, n_elem, d_vtss,
                                                                                 c.vert_tss);
    if (c.n_vert > 0) {
      k_vertex_min_init<<<grid_for(c.n_vert, 256), 256, 0, c.stream>>>(c.vmax, c.n_vert);
      k_vertex_min<ND><<<grid_for((long)n_elem*S::nvert, 256), 256, 0, c.stream>>>(c.vert_id, n_elem, c.vert_tss, c.vmax);
      k_vertex_gather<ND><<<grid_for((long)n_elem*S::nvert, 256), 256, 0, c.stream>>>(c.vert_id, n_elem, c.vmax,
                                                                                    c.vert_tss);
    }
  }

  // Solver::is_admissible (src/Solver.cpp:921-959); record [n_elem] and status[0] cleared first
  static void admissible(Ctx& c, int* record)
  {
    const int n_elem = c.n_car + c.n_def;
    cudaMemsetAsync(record, 0, (size_t)n_elem*sizeof(int), c.stream);
    cudaMemsetAsync(c.status, 0, sizeof(int), c.stream);
    const long total = (long)n_elem*(S::nq + 2*ND*S::nfq) + (long)c.n_ref*4*S::nfq;
    ProfScope ps(c, "admissible");
    k_admissible<ND, RS, FaceT><<<grid_for(total, 256), 256, 0, c.stream>>>(dev(c), record, c.status);
  }

  template <bool DEF>
  static void reconcile(Ctx& c, int cr, int uf)
  {
    const int e_begin = DEF ? c.n_car : 0;
    const int e_end = DEF ? c.n_car + c.n_def : c.n_car;
    if (e_end <= e_begin) return;
    const int blocks = (e_end - e_begin + S::epb - 1)/S::epb;
    constexpr size_t smem = ReconcileSmem<ND, RS, R, DEF>::bytes;
    auto kern = k_reconcile_ldg<ND, RS, R, DEF, FaceT>;
    static bool configured = false;
    if (!configured) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      configured = true;
    }
    ProfScope ps(c, DEF ? "reconcile_ldg_def" : "reconcile_ldg_car");
    const Tab<RS> t = tab(c);
    kern<<<blocks, S::threads, smem, c.stream>>>(dev(c), t, make_rowtab<RS, R>(t), e_begin, e_end, cr, uf);
  }

  template <bool VISC>
  static void neighbor(Ctx& c, bool fuse_bc)
  {
    const int block = c.face_threads;
    // one launch for small Cartesian meshes, where launch latency dominates; large ones keep
    // the leaner Cartesian kernel (the fused one carries the boundary code's registers)
    if (c.n_car_con && c.n_bc_con && !c.n_def_con && (long)c.n_car_con*S::nfq <= 2L*152*block) {
      const int car_blocks = grid_for((long)c.n_car_con*S::nfq, block);
      const int blocks = car_blocks + grid_for((long)c.n_bc_con*S::nfq, bc_warp);
      ProfScope ps(c, "neighbor_car_bc");
      if (fuse_bc) k_neighbor_car_bc<ND, RS, R, VISC, true, FaceT><<<blocks, block, 0, c.stream>>>(dev(c), car_blocks);
      else k_neighbor_car_bc<ND, RS, R, VISC, false, FaceT><<<blocks, block, 0, c.stream>>>(dev(c), car_blocks);
      return;
    }
    if (c.n_car_con) {
      ProfScope ps(c, "neighbor_car");
      k_neighbor<ND, RS, R, false, VISC, FaceT><<<grid_for((long)c.n_car_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
    }
    if (c.n_def_con) {
      ProfScope ps(c, "neighbor_def");
      k_neighbor<ND, RS, R, true, VISC, FaceT><<<grid_for((long)c.n_def_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
    }
    if (c.n_bc_con) {
      ProfScope ps(c, fuse_bc ? "neighbor_bc_fused" : "neighbor_bc");
      if (fuse_bc) k_bc_neighbor<ND, RS, R, VISC, true, FaceT><<<grid_for((long)c.n_bc_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
      else k_bc_neighbor<ND, RS, R, VISC, false, FaceT><<<grid_for((long)c.n_bc_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
    }
  }

  static void refine(Ctx& c, bool prolong, bool scale, bool offset)
  {
    if (!c.n_ref) return;
    ProfScope ps(c, prolong ? "prolong" : "restrict");
    if (prolong) k_refine<ND, RS, true, FaceT><<<c.n_ref, 256, 0, c.stream>>>(dev(c), tab(c), scale, offset);
    else k_refine<ND, RS, false, FaceT><<<c.n_ref, 256, 0, c.stream>>>(dev(c), tab(c), scale, offset);
  }

  static void bc_state(Ctx& c)
  {
    ProfScope ps(c, "bc_state");
    if (c.n_bc_con) k_bc_state<ND, RS, FaceT><<<grid_for((long)c.n_bc_con*S::nfq, 256), 256, 0, c.stream>>>(dev(c));
  }

  static void bc_flux(Ctx& c)
  {
    ProfScope ps(c, "bc_flux");
    if (c.n_bc_con) k_bc_flux<ND, RS, FaceT><<<grid_for((long)c.n_bc_con*S::nfq, 256), 256, 0, c.stream>>>(dev(c));
  }

  static void neighbor_reconcile(Ctx& c, bool fuse_bc)
  {
    const int block = c.face_threads;
    if (c.n_car_con) {
      ProfScope ps(c, "neighbor_reconcile_car");
      k_neighbor_reconcile<ND, RS, R, 0, false, FaceT><<<grid_for((long)c.n_car_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
    }
    if (c.n_def_con) {
      ProfScope ps(c, "neighbor_reconcile_def");
      k_neighbor_reconcile<ND, RS, R, 1, false, FaceT><<<grid_for((long)c.n_def_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
    }
    if (c.n_bc_con) {
      ProfScope ps(c, fuse_bc ? "neighbor_reconcile_bc_fused" : "neighbor_reconcile_bc");
      if (fuse_bc) k_neighbor_reconcile<ND, RS, R, 2, true, FaceT><<<grid_for((long)c.n_bc_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
      else k_neighbor_reconcile<ND, RS, R, 2, false, FaceT><<<grid_for((long)c.n_bc_con*S::nfq, block), block, 0, c.stream>>>(dev(c));
    }
  }

  // compute_euler (src/kernels_convective.cpp:8-19). fuse_bc: apply the state BCs inside
  // the boundary part of Neighbor (used by the solver layer, which would otherwise run
  // Solver::apply_state_bcs immediately before).
  static void compute_euler(Ctx& c, int stage, int cr, int uf, bool fuse_bc, const LocalDt& ldt)
  {
    hexed_transport inv{0., 0., 1., 1., 0};
    neighbor<false>(c, fuse_bc);
    refine(c, false, true, false);
    local<false, false>(c, stage, cr, uf, inv, inv, ldt);
    local<true, false>(c, stage, cr, uf, inv, inv, ldt);
    refine(c, true, false, false);
  }

  // compute_navier_stokes (src/kernels_diffusive.cpp:8-32) with the flux BCs on the device
  static void compute_navier_stokes(Ctx& c, int stage, int cr, int uf, const hexed_transport& visc,
                                    const hexed_transport& cond, bool fuse_bc)
  {
    neighbor<true>(c, fuse_bc);
    refine(c, false, true, false);
    refine(c, false, false, true);
    local<false, true>(c, stage, cr, uf, visc, cond);
    local<true, true>(c, stage, cr, uf, visc, cond);
    if (!stage) {
      refine(c, true, true, true);
      neighbor_reconcile(c, true);   // flux BCs fused into the boundary part
      refine(c, false, true, true);
      reconcile<false>(c, cr, uf);
      reconcile<true>(c, cr, uf);
    }
    refine(c, true, false, false);
  }

  static void max_dt(Ctx& c, double msc, double msd, int local_time, int viscous, const hexed_transport& visc,
                     const hexed_transport& cond, double max_time_step, double cheby)
  {
    // At most 16 CTAs per SM, each looping over its points: on the 32^3 row-size-6 mesh
    // (7.1 M points) this took the float kernel from 0.205 to 0.168 ms and the double one from
    // 1.49 to 1.42 ms against one CTA per 256 points (19,456 CTAs taking the ticket, and the
    // last one reading as many partials). Caps of 4 to 32 CTAs per SM measured within 4%.
    const long total = (long)(c.n_car + c.n_def)*S::nq;
    const int grid = grid_for(total, 256, std::min(152*16, c.max_partials));
    {
      ProfScope ps(c, "max_dt");
      const R icc = R(inv_cfl_conv(c, msc)), icd = R(inv_cfl_diff(c, msd));
      if (viscous) k_max_dt<ND, RS, R, true, FaceT><<<grid, 256, 0, c.stream>>>(dev(c), tab(c), icc, icd, local_time, make_tm<R>(visc), make_tm<R>(cond), c.partials, c.dt_ticket, max_time_step, cheby);
      else k_max_dt<ND, RS, R, false, FaceT><<<grid, 256, 0, c.stream>>>(dev(c), tab(c), icc, icd, local_time, make_tm<R>(visc), make_tm<R>(cond), c.partials, c.dt_ticket, max_time_step, cheby);
    }
  }

  static void write_face(Ctx& c, int e_begin, int n_elem)
  {
    const long total = (long)n_elem*ND*S::nv*S::nfq;
    if (total == 0) return;
    ProfScope ps(c, "write_face");
    k_write_face<ND, RS, FaceT><<<grid_for(total, 256), 256, 0, c.stream>>>(dev(c), tab(c), e_begin, n_elem);
  }

  static void residual_norm(Ctx& c, double* d_out)
  {
    const long total = (long)(c.n_car + c.n_def)*S::nq;
    const int grid = grid_for(total, 256, c.max_partials/S::nv);
    {
      ProfScope ps(c, "residual_partial");
      k_residual_partial<ND, RS, FaceT><<<grid, 256, 0, c.stream>>>(dev(c), tab(c), c.partials);
    }
    ProfScope ps(c, "residual_final");
    k_residual_final<S::nv><<<1, 32, 0, c.stream>>>(c.partials, grid, d_out);
  }

  // Solver::set_art_visc_admis (src/Solver.cpp:636-658)
  static void set_art_visc_admis(Ctx& c, double char_speed)
  {
    const int n_elem = c.n_car + c.n_def;
    if (n_elem == 0) return;   // k_av_uncert's grid would be empty
    {
      ProfScope ps(c, "av_uncert");
      k_av_uncert<ND, RS, R><<<(n_elem + av_warps - 1)/av_warps, av_warps*32, 0, c.stream>>>(c.elem, c.nom_size, n_elem, av_tab(c),
                                                                                  char_speed, av_ramp(), c.uncert);
    }
    cudaMemsetAsync(c.vmax, 0, sizeof(double)*c.n_vert, c.stream);
    {
      ProfScope ps(c, "av_vertex_max");
      k_av_vertex_max<ND><<<grid_for((long)n_elem*S::nvert, 256), 256, 0, c.stream>>>(c.vert_id, n_elem, c.uncert, c.vmax);
    }
    ProfScope ps(c, "av_interp");
    k_av_interp<ND, RS, R><<<grid_for((n_elem + S::epb - 1)/S::epb, 1), S::threads, 0, c.stream>>>(c.elem, c.vert_id, n_elem, av_tab(c), c.vmax);
  }

  // Solver::fix_admissibility's coefficient set-up (src/Solver.cpp:990-1039): the elements'
  // admissibility records to a vertex maximum, the element maximum of that back to its
  // vertices, interpolated into the Laplacian artificial-viscosity row, then the bulk and
  // Laplacian rows swapped. swap_only: only the swap back (src/Solver.cpp:1083-1089). Without
  // a vertex table the coefficient is not formed (the rows are swapped all the same).
  static void fix_admis_coef(Ctx& c, const int* d_record, bool swap_only)
  {
    const int n_elem = c.n_car + c.n_def;
    if (!swap_only && c.n_vert > 0) {
      ProfScope ps(c, "fix_admis_coef");
      k_record_to_value<<<grid_for(n_elem, 256), 256, 0, c.stream>>>(d_record, n_elem, c.uncert);
      cudaMemsetAsync(c.vmax, 0, sizeof(double)*c.n_vert, c.stream);
      k_av_vertex_max<ND><<<grid_for((long)n_elem*S::nvert, 256), 256, 0, c.stream>>>(c.vert_id, n_elem, c.uncert, c.vmax);
      k_elem_vertex_max<ND><<<grid_for(n_elem, 256), 256, 0, c.stream>>>(c.vert_id, n_elem, c.vmax, c.uncert);
      cudaMemsetAsync(c.vmax, 0, sizeof(double)*c.n_vert, c.stream);
      k_av_vertex_max<ND><<<grid_for((long)n_elem*S::nvert, 256), 256, 0, c.stream>>>(c.vert_id, n_elem, c.uncert, c.vmax);
      k_av_interp<ND, RS, R><<<grid_for((n_elem + S::epb - 1)/S::epb, 1), S::threads, 0, c.stream>>>(c.elem, c.vert_id, n_elem, av_tab(c), c.vmax);
    }
    k_swap_av<ND, RS><<<grid_for((long)n_elem*S::nq, 256), 256, 0, c.stream>>>(c.elem, n_elem);
  }

  // RefState terms of every element, after the reference state changed (mixed form)
  static void ref_terms(Ctx& c)
  {
    static_assert(sizeof(RefState<ND, float>) == (3*ND + 7 + 3)/4*4*sizeof(float),
                  "ref_terms rows are 3 nd + 7 floats, padded to 16 bytes");
    const int n = c.cap_car + c.n_def;
    if (c.ref_state && c.ref_terms && n > 0)
      k_ref_terms<ND><<<grid_for(n, 256), 256, 0, c.stream>>>(c.ref_state, n, reinterpret_cast<RefState<ND, float>*>(c.ref_terms));
  }

  static void segment_residual_norms(Ctx& c, int n_seg, const int* d_begin, const int* d_count, double* d_out)
  {
    ProfScope ps(c, "segment_residual");
    k_segment_residual<ND, RS, FaceT><<<n_seg, 256, 0, c.stream>>>(dev(c), tab(c), d_begin, d_count, d_out);
  }

  // ---------------------------------------------------------------- smoothness-based AV
  static SavDev sav_dev(Ctx& c)
  {
    SavDev m;
    m.n_car = c.n_car; m.n_elem = c.n_car + c.n_def; m.n_car_con = c.n_car_con; m.n_def_con = c.n_def_con;
    m.n_bc_con = c.n_bc_con; m.n_ref = c.n_ref;
    m.elem = c.elem; m.aux = c.sav_aux; m.face = c.sav_face;
    m.nom_size = c.nom_size; m.vert_tss = c.vert_tss; m.jac = c.jac; m.face_nrml = c.face_nrml;
    m.car_con = c.car_con; m.def_con = c.def_con; m.def_con_nrml = c.def_con_nrml;
    m.bc_con = c.bc_con; m.bc_nrml = c.bc_nrml; m.ref_face = c.ref_face; m.bc_spec = c.bc_spec;
    m.partials = c.sav_partials;
    return m;
  }

  static int sav_slot_dof() { return SavShape<ND, RS>::slot_dof; }

  template <int NVAR>
  static void sav_refine(Ctx& c, const SavDev& m, const Tab<RS>& t, bool prolong, bool scale, bool offset)
  {
    if (!c.n_ref) return;
    if (prolong) k_sav_refine<ND, RS, true, NVAR><<<c.n_ref, 256, 0, c.stream>>>(m, t, scale, offset);
    else k_sav_refine<ND, RS, false, NVAR><<<c.n_ref, 256, 0, c.stream>>>(m, t, scale, offset);
  }

  // Runs body(0), ..., body(n - 1), where body(i) enqueues the same launches for every i >= 1.
  // From the second iteration on, the launches of one iteration are captured once as a CUDA
  // graph and the graph is launched for the rest: a pseudo-time loop of thousands of
  // iterations on a small mesh is otherwise bound by launch latency. Eager throughout when
  // the per-kernel profiler is on (so that it sees every kernel), inside another capture, for
  // fewer than three iterations, or if a graph call fails (from that iteration on).
  template <typename F>
  static void repeat_iterations(Ctx& c, int n, F&& body)
  {
    const bool eager = n < 3 || c.capturing || (c.prof && c.prof->enabled);
    int i = 0;
    if (!eager) {
      body(i++);
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      bool failed = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess;
      if (!failed) {
        c.capturing = true;
        body(1);   // recorded, not run
        c.capturing = false;
        failed = cudaStreamEndCapture(c.stream, &graph) != cudaSuccess || !graph ||
                 cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess;
        for (; !failed && i < n; ++i) failed = cudaGraphLaunch(exec, c.stream) != cudaSuccess;
        if (graph) cudaGraphDestroy(graph);
        if (exec) cudaGraphExecDestroy(exec);   // freed once its launches complete
      }
      if (failed) cudaGetLastError();   // the graph call's error; the eager loop runs the rest
    }
    for (; i < n; ++i) body(i);
  }

  // Solver::update_art_visc_smoothness (src/Solver.cpp:457-582) with Solver::diffuse_art_visc
  // (src/Solver.cpp:428-455): the reference's kernel sequence, then the flow's Write_face and
  // Prolong (src/Solver.cpp:577-578). d_residual receives art_visc_residual.
  static void update_art_visc_smoothness(Ctx& c, const hexed_sav_params& p, double* d_residual)
  {
    using SS = SavShape<ND, RS>;
    constexpr int nq = SS::nq;
    const SavDev m = sav_dev(c);
    const Tab<RS> t = tab(c);
    const SavTab<RS> st = make_savtab<RS>(t);
    const int n_elem = m.n_elem;
    const long n_pts = (long)n_elem*nq;
    const int g_pts = grid_for(n_pts, 256);
    const long n_face_pts = (long)(m.n_car_con + m.n_def_con + m.n_bc_con)*SS::nfq;
    const int g_con = grid_for(n_face_pts, 256);
    constexpr int blk = SS::block;   // the volume kernels' launch bound
    constexpr size_t smem_adv = SavAdvSmem<ND, RS>::bytes;
    constexpr size_t smem_diff = SavDiffSmem<ND, RS>::bytes;
    static bool configured = false;
    if (!configured) {
      cudaFuncSetAttribute(k_sav_local_advection<ND, RS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_adv);
      cudaFuncSetAttribute(k_sav_local_diffusion<ND, RS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_diff);
      configured = true;
    }
    auto sav_faces = [&](int mode) {
      const long n = (long)n_elem*ND*SS::nfq*(mode ? SS::n_sav : SS::n_adv_extrap);
      ProfScope ps(c, "sav_write_face");
      k_sav_write_face<ND, RS><<<grid_for(n, 256), 256, 0, c.stream>>>(m, st, mode);
    };
    {
      ProfScope ps(c, "sav_setup");
      // advection velocity, then Max_dt of pde::Advection with local time stepping
      k_sav_velocity<ND, RS><<<g_pts, 256, 0, c.stream>>>(m);
      k_sav_max_dt<ND, RS><<<g_pts, 256, 0, c.stream>>>(m, st, 0, t.max_cfl*p.advect_safety);
    }
    repeat_iterations(c, p.advect_iters, [&](int iter) {
      // compute_write_face_advection + compute_prolong_advection; after the first iteration the
      // previous stage's volume kernel and prolongation have written these same traces
      if (iter == 0) {
        sav_faces(0);
        sav_refine<SS::n_adv_extrap>(c, m, t, true, false, false);
      }
      for (int stage = 0; stage < 2; ++stage) {
        if (n_face_pts) {   // boundary ghosts included (sav_bc_advection_point)
          ProfScope ps(c, "sav_neighbor_advection");
          k_sav_neighbor_advection<ND, RS><<<g_con, 256, 0, c.stream>>>(m, st);
        }
        sav_refine<SS::n_adv_extrap>(c, m, t, false, true, false);
        {
          ProfScope ps(c, "sav_local_advection");
          // Local with its Write_face of the new advection traces
          k_sav_local_advection<ND, RS><<<n_elem, blk, smem_adv, c.stream>>>(m, st, stage, p.advect_length,
                                                                            t.step_ratio);
        }
        sav_refine<SS::n_adv_extrap>(c, m, t, true, false, false);
      }
    });
    // projection onto the Legendre mode of degree av_rs - 1
    AvTab<RS, double> wo;
    for (int i = 0; i < RS; ++i) {
      wo.w[i] = t.weight[i];
      wo.ow[i] = c.tables.ortho[(p.av_row_size - 1)*RS + i];
      wo.node[i] = t.node[i];
    }
    // diffuse_art_visc: n_forcing - 1 = 3 real steps of pde::Smooth_art_visc at once
    const double diff_time = p.diff_ratio*p.advect_length*p.advect_length/(SS::n_forcing - 1);
    {
      ProfScope ps(c, "sav_setup");
      k_sav_project<ND, RS><<<g_pts, 256, 0, c.stream>>>(m, wo);
      k_sav_max_dt<ND, RS><<<g_pts, 256, 0, c.stream>>>(m, st, 1, -2/t.min_eig_diffusion*p.diff_safety);
    }
    sav_faces(1);
    sav_refine<SS::nv>(c, m, t, true, false, false);   // compute_prolong: the flow's nv variables
    repeat_iterations(c, p.diff_iters, [&](int) {
      for (int i_cheby = 0; i_cheby < p.n_cheby; ++i_cheby) {
        // math::chebyshev_step (src/math.cpp:104-107)
        const double s = 1/(1 - std::cos((p.n_cheby - i_cheby - 0.5)*3.14159265358979323846/p.n_cheby));
        if (n_face_pts) {   // boundary ghosts included (sav_bc_diffusion_point)
          ProfScope ps(c, "sav_neighbor_ldg");
          k_sav_neighbor_ldg<ND, RS><<<g_con, 256, 0, c.stream>>>(m, 0);
        }
        sav_refine<SS::n_sav>(c, m, t, false, true, false);
        sav_refine<SS::n_sav>(c, m, t, false, false, true);
        {
          ProfScope ps(c, "sav_local_diffusion");
          k_sav_local_diffusion<ND, RS><<<n_elem, blk, smem_diff, c.stream>>>(m, st, s, diff_time);
        }
        sav_refine<SS::n_sav>(c, m, t, true, true, true);
        if (n_face_pts) {
          ProfScope ps(c, "sav_neighbor_ldg");
          k_sav_neighbor_ldg<ND, RS><<<g_con, 256, 0, c.stream>>>(m, 1);
        }
        sav_refine<SS::n_sav>(c, m, t, false, true, true);
        {
          ProfScope ps(c, "sav_reconcile");
          k_sav_reconcile<ND, RS><<<g_pts, 256, 0, c.stream>>>(m, st, s, diff_time, s);
        }
        sav_faces(1);
        sav_refine<SS::n_sav>(c, m, t, true, false, false);
      }
    });
    // coefficient, residual, momentum put back; then the flow's traces
    const double mult = p.visc_mult*p.advect_length;
    const double us_max = p.advect_length*p.unscaled_max*std::sqrt(2*p.freestream_energy/p.freestream_mass);
    {
      ProfScope ps(c, "sav_setup");
      k_sav_finish<ND, RS><<<grid_for(n_elem, 1), 128, 0, c.stream>>>(m, wo, mult, us_max);
      k_sav_residual<<<1, 256, 0, c.stream>>>(m.partials, n_elem, d_residual);
    }
    write_face(c, 0, n_elem);
    refine(c, true, false, false);
  }

  static const OpsTable* table()
  {
    static const OpsTable t = {
      compute_euler, compute_navier_stokes, max_dt, refine, write_face, bc_state, bc_flux, residual_norm,
      set_art_visc_admis, segment_residual_norms, local_elems_per_cta, admissible, compute_jacobian,
      fix_admis_coef, ref_terms, update_art_visc_smoothness, sav_slot_dof,
    };
    return &t;
  }
};

} // namespace hx

#define HEXED_INSTANTIATE(ND, RS) \
  namespace hx { \
  const OpsTable* ops_##ND##_##RS(int precision) \
  { \
    return precision == HEXED_MIXED ? Runner<ND, RS, float>::table() : Runner<ND, RS, double>::table(); \
  } \
  }
