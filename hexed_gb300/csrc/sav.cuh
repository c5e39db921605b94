// sav.cuh -- smoothness-based artificial viscosity on the device (FP64):
// Solver::update_art_visc_smoothness (src/Solver.cpp:457-582) and Solver::diffuse_art_visc
// (src/Solver.cpp:428-455), the Spatial kernels applied to pde::Advection and
// pde::Smooth_art_visc (include/pde.hpp:265-431).
//
// Storage beside the arena (allocated on first use, kept between calls like the reference's
// element storage):
//  * aux  [n_elem][4 + 2 rs][nq]: the four art_visc_forcing rows (Storage_params::n_forcing),
//    the advection state (rs rows, 1 at creation as Solver's constructor sets it,
//    src/Solver.cpp:201-211) and its residual cache (rs rows);
//  * face [n_slot][slot_dof], slot_dof = max(2 nv, nd + rs) nfq: one slot per arena slot, the
//    size of a reference Face_connection face (include/connection.hpp:58-66), LDG half at
//    nv nfq as in Element::face (src/Element.cpp:189). The reference keeps these traces in the
//    flow's face storage; here they have their own, so the flow's traces are untouched.
// The flow state is used in place as the reference does: momentum is divided by sqrt(2 rho E)
// (the advection velocity) and multiplied back at the end; the time-step-scale row holds the
// pseudo-time steps; the bulk AV row receives the coefficient.
//
// Every kernel is FP64 with one thread per quadrature point (volume) or face point (faces):
// an advection stage moves nd + 3 rs rows per element and its traces, and is bound by HBM like
// the flow's inviscid kernel; the diffusion stages move 3-row fields.
#pragma once
#include "kernels.cuh"

namespace hx {

// Double views of the arena and of the smoothness-AV storage (both precision forms keep the
// double metrics and normals beside their float copies).
struct SavDev {
  int n_car, n_elem, n_car_con, n_def_con, n_bc_con, n_ref;
  double* elem;
  double* aux;
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
  const int* ref_face;
  const hexed_bc_spec* bc_spec;
  double* partials;
};

template <int ND, int RS>
struct SavShape {
  static constexpr int nq = ipow(RS, ND), nfq = nq/RS, nv = ND + 2, nvert = 1 << ND;
  static constexpr int n_forcing = 4;
  static constexpr int n_adv = RS;                       // Storage_params::n_advection
  static constexpr int n_aux = n_forcing + 2*n_adv;
  static constexpr int n_adv_extrap = ND + n_adv;        // pde::Advection::n_extrap
  static constexpr int n_sav = 3;                        // pde::Smooth_art_visc::n_extrap
  static constexpr int slot_dof = (2*nv > n_adv_extrap ? 2*nv : n_adv_extrap)*nfq;
  // threads of the per-element volume kernels: one per quadrature point, whole warps, >= 64
  static constexpr int block = (nq + 31)/32*32 < 64 ? 64 : (nq + 31)/32*32;
  static __device__ __forceinline__ double* forcing(const SavDev& m, int e) { return m.aux + (size_t)e*n_aux*nq; }
  static __device__ __forceinline__ double* adv(const SavDev& m, int e) { return forcing(m, e) + n_forcing*nq; }
  static __device__ __forceinline__ double* adv_cache(const SavDev& m, int e) { return adv(m, e) + n_adv*nq; }
  static __device__ __forceinline__ double* slot(const SavDev& m, int s, bool ldg)
  {
    return m.face + (size_t)s*slot_dof + (ldg ? nv*nfq : 0);
  }
  // quadrature point of node i of row i_fq along dimension d (include/Row_index.hpp)
  static __device__ __forceinline__ int row_qpoint(int d, int i_fq, int i)
  {
    const int stride = ipow(RS, ND - 1 - d);
    return (i_fq/stride)*stride*RS + i_fq%stride + i*stride;
  }
};

// Row-local operators of Derivative (include/Derivative.hpp:22-60) and the advection nodes.
template <int RS>
struct SavTab {
  double diff[RS*RS], bound[2*RS], lift[RS*2], node[RS], adv_node[RS];
};

template <int RS>
inline SavTab<RS> make_savtab(const Tab<RS>& t)
{
  SavTab<RS> s;
  for (int i = 0; i < RS*RS; ++i) s.diff[i] = t.diff[i];
  for (int i = 0; i < 2*RS; ++i) { s.bound[i] = t.bound[i]; s.lift[i] = t.lift[i]; }
  for (int i = 0; i < RS; ++i) { s.node[i] = t.node[i]; s.adv_node[i] = 2*t.node[i] - 1.; }   // pde.hpp:281
  return s;
}

// math::interp of the vertex time-step scales at a qpoint (include/math.hpp:207-218)
template <int ND, int RS>
__device__ __forceinline__ double sav_spacing(const SavDev& m, const SavTab<RS>& t, int e, int q)
{
  constexpr int nvert = 1 << ND;
  double vals[nvert];
  #pragma unroll
  for (int i = 0; i < nvert; ++i) vals[i] = m.vert_tss[(size_t)e*nvert + i];
  int stride = nvert;
  #pragma unroll
  for (int d = 0; d < ND; ++d) {
    const double coord = t.node[(q/ipow(RS, ND - 1 - d))%RS];
    stride /= 2;
    for (int i = 0; i < stride; ++i) vals[i] += coord*(vals[i + stride] - vals[i]);
  }
  return vals[0];
}

// Momentum over sqrt(2 rho E): the advection velocity (Solver.cpp:468-478).
template <int ND, int RS>
__global__ void k_sav_velocity(SavDev m)
{
  using S = SavShape<ND, RS>;
  const long total = (long)m.n_elem*S::nq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int e = int(t/S::nq), q = int(t%S::nq);
    double* st = m.elem + (size_t)e*(S::nv + 3)*S::nq;
    const double scale = sqrt(2*st[ND*S::nq + q]*st[(ND + 1)*S::nq + q]);
    #pragma unroll
    for (int d = 0; d < ND; ++d) st[d*S::nq + q] /= scale;
  }
}

// Local time step of pde::Advection (char speed max(1, |v|), pde.hpp:343-346) or of
// pde::Smooth_art_visc (diffusivity 1): Spatial::Max_dt with local time stepping
// (include/Spatial.hpp:784-828). max_cfl = max_cfl_c (advection) or max_cfl_d (diffusion).
template <int ND, int RS>
__global__ void k_sav_max_dt(SavDev m, SavTab<RS> tab, int diffusion, double max_cfl)
{
  using S = SavShape<ND, RS>;
  const long total = (long)m.n_elem*S::nq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int e = int(t/S::nq), q = int(t%S::nq);
    double* st = m.elem + (size_t)e*(S::nv + 3)*S::nq;
    const double sp = sav_spacing<ND, RS>(m, tab, e, q);
    double scale = 0;
    if (diffusion) {
      scale += 1./max_cfl/sp/sp;
    } else {
      double sq = 0.;
      #pragma unroll
      for (int d = 0; d < ND; ++d) sq += st[d*S::nq + q]*st[d*S::nq + q];
      const double cs = fmax(1., sqrt(sq));
      scale += cs/max_cfl/sp;
    }
    st[S::nv*S::nq + q] = 1./scale;
  }
}

// Spatial::Write_face (include/Spatial.hpp:41-57) into the smoothness-AV slots: mode 0 the
// Advection traces (velocity rows, then the advection state; pde.hpp:284-290), mode 1 the
// Smooth_art_visc traces (forcing rows 1-3; pde.hpp:372-377). One thread per (element,
// dimension, face point, variable) writes both faces of its row.
template <int ND, int RS>
__global__ void k_sav_write_face(SavDev m, SavTab<RS> tab, int mode)
{
  using S = SavShape<ND, RS>;
  const int n_var = mode ? S::n_sav : S::n_adv_extrap;
  const long total = (long)m.n_elem*ND*S::nfq*n_var;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int v = int(t%n_var);
    long r = t/n_var;
    const int i_fq = int(r%S::nfq);
    r /= S::nfq;
    const int d = int(r%ND), e = int(r/ND);
    const double* row;
    if (mode) row = S::forcing(m, e) + (1 + v)*S::nq;
    else if (v < ND) row = m.elem + ((size_t)e*(S::nv + 3) + v)*S::nq;
    else row = S::adv(m, e) + (v - ND)*S::nq;
    double x[RS];
    #pragma unroll
    for (int i = 0; i < RS; ++i) x[i] = row[S::row_qpoint(d, i_fq, i)];
    #pragma unroll
    for (int s = 0; s < 2; ++s) {
      double acc = 0.;
      #pragma unroll
      for (int i = 0; i < RS; ++i) acc += tab.bound[s*RS + i]*x[i];
      S::slot(m, e*2*ND + 2*d + s, false)[v*S::nfq + i_fq] = acc;
    }
  }
}

// Prolong_refined / Restrict_refined of NVAR variables of the smoothness-AV slots.
template <int ND, int RS, bool PROLONG, int NVAR>
__global__ void k_sav_refine(SavDev m, Tab<RS> tab, int scale, int offset)
{
  using S = SavShape<ND, RS>;
  refine_face<ND, RS, PROLONG, NVAR, double>(m.face, S::slot_dof, S::nv*S::nfq, m.ref_face + 7*blockIdx.x, tab,
                                             scale, offset);
}

// Flow_bc::apply_advection and its overrides (src/Boundary_condition.cpp:24-41, 346-368,
// 429-448, 460-463) at face point q of boundary connection i: the ghost from the inside at the
// same point. Run by k_sav_neighbor_advection's thread for that point just before its flux
// (a boundary connection's faces are not permuted), so it needs no launch of its own.
template <int ND, int RS>
__device__ __forceinline__ void sav_bc_advection_point(const SavDev& m, int i, int q)
{
  using S = SavShape<ND, RS>;
  constexpr int nfq = S::nfq;
  {
    const int* c = m.bc_con + 4*i;
    const hexed_bc_spec& b = m.bc_spec[c[3]];
    const double* in = S::slot(m, c[0], false);
    double* gh = S::slot(m, c[1], false);
    switch (b.kind) {
      case HEXED_BC_NONPENETRATION: {
        const double* nrml = m.bc_nrml + (size_t)i*ND*nfq;
        double dot = 0., nsq = 0.;
        #pragma unroll
        for (int d = 0; d < ND; ++d) {
          const double n = nrml[d*nfq + q];
          dot += in[d*nfq + q]*n;
          nsq += n*n;
        }
        #pragma unroll
        for (int d = 0; d < ND; ++d) gh[d*nfq + q] = in[d*nfq + q] - 2*dot*nrml[d*nfq + q]/nsq;
        for (int a = 0; a < S::n_adv; ++a) gh[(ND + a)*nfq + q] = in[(ND + a)*nfq + q];
        break;
      }
      case HEXED_BC_NO_SLIP:
        #pragma unroll
        for (int d = 0; d < ND; ++d) gh[d*nfq + q] = -in[d*nfq + q];
        for (int a = 0; a < S::n_adv; ++a) gh[(ND + a)*nfq + q] = in[(ND + a)*nfq + q];
        break;
      case HEXED_BC_COPY:
        // copy_state (src/Boundary_condition.cpp:12-22): both halves of the face, nv nfq each
        for (int k = 0; k < 2*S::nv; ++k) gh[k*nfq + q] = in[k*nfq + q];
        break;
      default:
        // velocity as inside; advected scalars mirrored about 1
        #pragma unroll
        for (int d = 0; d < ND; ++d) gh[d*nfq + q] = in[d*nfq + q];
        for (int a = 0; a < S::n_adv; ++a) gh[(ND + a)*nfq + q] = 2. - in[(ND + a)*nfq + q];
    }
  }
}

// Connection i of the concatenated lists (Cartesian, deformed, boundary): its slots, packed
// direction and normal (null for Cartesian), with the direction encoding of Neighbor.
__device__ __forceinline__ const double* sav_connection(const SavDev& m, int nd, int nfq, int i, int& s0, int& s1,
                                                        int& dir)
{
  if (i < m.n_car_con) {
    const int* c = m.car_con + 3*i;
    s0 = c[0]; s1 = c[1]; dir = c[2] | (c[2] << 2) | (1 << 4);
    return nullptr;
  }
  i -= m.n_car_con;
  if (i < m.n_def_con) {
    const int* c = m.def_con + 3*i;
    s0 = c[0]; s1 = c[1]; dir = c[2];
    return m.def_con_nrml + (size_t)i*nd*nfq;
  }
  i -= m.n_def_con;
  const int* c = m.bc_con + 4*i;
  s0 = c[0]; s1 = c[1]; dir = bc_dir(c[2]);
  return m.bc_nrml + (size_t)i*nd*nfq;
}

// Spatial<pde::Advection>::Neighbor (include/Spatial.hpp:613-705): local Lax-Friedrichs flux
// of the advected scalars, written over the first rs face variables of both sides.
template <int ND, int RS>
__global__ void k_sav_neighbor_advection(SavDev m, SavTab<RS> tab)
{
  using S = SavShape<ND, RS>;
  constexpr int nfq = S::nfq, n_adv = S::n_adv, n_ex = S::n_adv_extrap;
  const long total = (long)(m.n_car_con + m.n_def_con + m.n_bc_con)*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    int s0, s1, dir;
    const double* nrml = sav_connection(m, ND, nfq, int(t/nfq), s0, s1, dir);
    const int q = int(t%nfq);
    const int i_bc = int(t/nfq) - m.n_car_con - m.n_def_con;
    if (i_bc >= 0) sav_bc_advection_point<ND, RS>(m, i_bc, q);   // the ghost first
    const bool deformed = nrml != nullptr;
    int sign0 = 1, sign1 = 1;
    if (deformed) {
      sign0 = 1 - 2*(((dir >> 4) & 1) == 0);
      sign1 = 1 - 2*(((dir >> 5) & 1) == 1);
    }
    const int q1 = deformed ? perm_index<ND, RS>(dir, q) : q;
    double* f0 = S::slot(m, s0, false);
    double* f1 = S::slot(m, s1, false);
    double n[ND];
    #pragma unroll
    for (int d = 0; d < ND; ++d) n[d] = deformed ? sign0*nrml[d*nfq + q] : (d == (dir & 3) ? 1. : 0.);
    double u0[n_ex], u1[n_ex];
    #pragma unroll
    for (int v = 0; v < n_ex; ++v) { u0[v] = f0[v*nfq + q]; u1[v] = f1[v*nfq + q1]; }
    double nv0 = 0., nv1 = 0., sq0 = 0., sq1 = 0.;
    #pragma unroll
    for (int d = 0; d < ND; ++d) { nv0 += u0[d]*n[d]; nv1 += u1[d]*n[d]; }
    #pragma unroll
    for (int d = 0; d < ND; ++d) { sq0 += u0[d]*u0[d]; sq1 += u1[d]*u1[d]; }
    // max(max(1, |v0|), max(1, |v1|)) with one square root: sqrt is correctly rounded and
    // monotonic, and sqrt(1) = 1, so this is the same number
    const double cs = sqrt(fmax(1., fmax(sq0, sq1)));
    double nn = 0.;
    #pragma unroll
    for (int d = 0; d < ND; ++d) nn += n[d]*n[d];
    const double mult = cs*(deformed ? sqrt(nn) : 1.);   // Cartesian normals are unit vectors
    #pragma unroll
    for (int a = 0; a < n_adv; ++a) {
      const double fl0 = tab.adv_node[a]*nv0*u0[ND + a];
      const double fl1 = tab.adv_node[a]*nv1*u1[ND + a];
      const double flux = .5*(fl0 + fl1 + mult*(u0[ND + a] - u1[ND + a]));
      f0[a*nfq + q] = sign0*flux;
      f1[a*nfq + q1] = sign1*flux;
    }
  }
}

// acc + sign*(Derivative::operator() for output node i) of a row x whose boundary
// corrections bf_s = fb_s - B_s.x were formed once for the whole row (Derivative.hpp:50-55),
// sum_j diff[i][j] x_j + (lift[i][0] bf0 + lift[i][1] bf1), as one FMA chain into acc, lift
// terms first (each FP64 operation saved counts: these kernels are bound by the FP64 pipe).
template <int RS, int SIGN>
__device__ __forceinline__ double accumulate_derivative_bf(double acc, const SavTab<RS>& t, const double (&x)[RS],
                                                           double bf0, double bf1, int i)
{
  acc += SIGN*t.lift[i*2]*bf0;
  acc += SIGN*t.lift[i*2 + 1]*bf1;
  #pragma unroll
  for (int j = 0; j < RS; ++j) acc += SIGN*t.diff[i*RS + j]*x[j];
  return acc;
}

// Shared memory of k_sav_local_advection, in doubles: fluxes [nd][rs][nq], the per-row boundary
// corrections [nd][rs][nfq][2], and the rows whose traces the kernel writes ([nd + rs][nq]:
// velocity, then the new advection state).
template <int ND, int RS>
struct SavAdvSmem {
  using S = SavShape<ND, RS>;
  static constexpr int flux = 0;
  static constexpr int bf = ND*S::n_adv*S::nq;
  static constexpr int rows = bf + ND*S::n_adv*S::nfq*2;
  static constexpr size_t bytes = sizeof(double)*(size_t)(rows + S::n_adv_extrap*S::nq);
};

// Spatial<pde::Advection>::Local (include/Spatial.hpp:326-509): flux node_a (v.n_i) a_a, the
// source 2/advect_length in the first stage, and Advection::write_update (pde.hpp:292-300):
// pseudo = 1 + 2 tss/advect_length; the first stage sets a = (a + update)/pseudo, the second
// adds update/pseudo; then Write_face of the velocity and the new advection state
// (Spatial.hpp:507, pde::Advection::fetch_extrap). One CTA per element, one thread per
// quadrature point. The boundary corrections fb - B.f of each row are formed once per row (a
// task per row), not once per point: the kernel is bound by the FP64 pipe, and they were most
// of its work.
template <int ND, int RS>
__global__ void __launch_bounds__(SavShape<ND, RS>::block)
k_sav_local_advection(SavDev m, SavTab<RS> tab, int stage, double advect_length, double step_ratio)
{
  using S = SavShape<ND, RS>;
  using L = SavAdvSmem<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, n_adv = S::n_adv, n_ex = S::n_adv_extrap;
  extern __shared__ double s_mem[];
  double* s_flux = s_mem + L::flux;   // [ND][n_adv][nq]
  double* s_bf = s_mem + L::bf;       // [ND][n_adv][nfq][2]
  double* s_rows = s_mem + L::rows;   // [n_ex][nq]
  const int e = blockIdx.x;
  const int q = threadIdx.x;
  const bool deformed = e >= m.n_car;
  double* st = m.elem + (size_t)e*(S::nv + 3)*nq;
  double* a_st = S::adv(m, e);
  double* rcache = S::adv_cache(m, e);
  const double* nrml = deformed ? m.jac + (size_t)(e - m.n_car)*(ND*ND + 1)*nq : nullptr;
  const double d_pos = m.nom_size[e];
  double a_old[n_adv];
  if (q < nq) {
    double vel[ND];
    #pragma unroll
    for (int j = 0; j < ND; ++j) { vel[j] = st[j*nq + q]; s_rows[j*nq + q] = vel[j]; }
    #pragma unroll
    for (int a = 0; a < n_adv; ++a) a_old[a] = a_st[a*nq + q];
    #pragma unroll
    for (int i = 0; i < ND; ++i) {
      double nrml_veloc = 0;
      #pragma unroll
      for (int j = 0; j < ND; ++j) nrml_veloc += vel[j]*(deformed ? nrml[(i*ND + j)*nq + q] : (i == j ? 1. : 0.));
      #pragma unroll
      for (int a = 0; a < n_adv; ++a) s_flux[(i*n_adv + a)*nq + q] = tab.adv_node[a]*nrml_veloc*a_old[a];
    }
  }
  __syncthreads();
  // boundary corrections of every row: fb_s - B_s.f with the face fluxes of Neighbor
  for (int t = threadIdx.x; t < ND*n_adv*nfq; t += blockDim.x) {
    const int i_fq = t%nfq, a = (t/nfq)%n_adv, d = t/(nfq*n_adv);
    double x[RS];
    #pragma unroll
    for (int k = 0; k < RS; ++k) x[k] = s_flux[(d*n_adv + a)*nq + S::row_qpoint(d, i_fq, k)];
    double b0 = 0., b1 = 0.;
    #pragma unroll
    for (int j = 0; j < RS; ++j) { b0 += tab.bound[j]*x[j]; b1 += tab.bound[RS + j]*x[j]; }
    s_bf[2*t] = S::slot(m, e*2*ND + 2*d, false)[a*nfq + i_fq] - b0;
    s_bf[2*t + 1] = S::slot(m, e*2*ND + 2*d + 1, false)[a*nfq + i_fq] - b1;
  }
  __syncthreads();
  if (q < nq) {
    double rate[n_adv];
    #pragma unroll
    for (int a = 0; a < n_adv; ++a) rate[a] = 0.;
    #pragma unroll
    for (int d = 0; d < ND; ++d) {
      const int stride = ipow(RS, ND - 1 - d);
      const int i = (q/stride)%RS;
      const int i_fq = (q/(stride*RS))*stride + q%stride;
      #pragma unroll
      for (int a = 0; a < n_adv; ++a) {
        double x[RS];
        #pragma unroll
        for (int k = 0; k < RS; ++k) x[k] = s_flux[(d*n_adv + a)*nq + q - i*stride + k*stride];
        const int r = (d*n_adv + a)*nfq + i_fq;
        rate[a] = accumulate_derivative_bf<RS, -1>(rate[a], tab, x, s_bf[2*r], s_bf[2*r + 1], i);
      }
    }
    // three divisions per point (the element's size times the determinant, the pseudo-time
    // factor, 2/advect_length) and reciprocal multiplies after them: each FP64 division costs
    // about ten FP64 operations, and this kernel is bound by the FP64 pipe
    const double tss = st[S::nv*nq + q];
    const double det = deformed ? nrml[ND*ND*nq + q] : 1.;
    const double update_coef = stage ? 1.*step_ratio : 1.;
    const double mult = update_coef*tss/(deformed ? d_pos*det : d_pos);
    const double two_l = 2/advect_length;
    const double inv_pseudo = 1/(1 + tss*two_l);
    double src_mult = d_pos;
    if (deformed) src_mult *= det;
    const double source = src_mult*two_l;
    #pragma unroll
    for (int a = 0; a < n_adv; ++a) {
      double u = rate[a];
      if (stage) {
        u -= rcache[a*nq + q];
      } else {
        rcache[a*nq + q] = u;
        u += source;
      }
      u *= mult;
      const double x = a_old[a];
      const double nx = stage ? x + u*inv_pseudo : (x + u)*inv_pseudo;
      a_st[a*nq + q] = nx;
      s_rows[(ND + a)*nq + q] = nx;
    }
  }
  __syncthreads();
  // Write_face of the velocity and the new advection state (both faces of each row)
  for (int t = threadIdx.x; t < ND*n_ex*nfq; t += blockDim.x) {
    const int i_fq = t%nfq, v = (t/nfq)%n_ex, d = t/(nfq*n_ex);
    double x[RS];
    #pragma unroll
    for (int k = 0; k < RS; ++k) x[k] = s_rows[v*nq + S::row_qpoint(d, i_fq, k)];
    #pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      double acc = 0.;
      #pragma unroll
      for (int k = 0; k < RS; ++k) acc += tab.bound[s2*RS + k]*x[k];
      S::slot(m, e*2*ND + 2*d + s2, false)[v*nfq + i_fq] = acc;
    }
  }
}

// Solver.cpp:527-542: projection of the advection state onto the Legendre mode of degree
// av_rs - 1 (w[i] weight_i, ow[i] orthogonal(av_rs - 1)_i), into forcing row 0 as
// proj^2 * 2 E / rho.
template <int ND, int RS>
__global__ void k_sav_project(SavDev m, AvTab<RS, double> wo)
{
  using S = SavShape<ND, RS>;
  const long total = (long)m.n_elem*S::nq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int e = int(t/S::nq), q = int(t%S::nq);
    const double* a_st = S::adv(m, e);
    const double* st = m.elem + (size_t)e*(S::nv + 3)*S::nq;
    double proj = 0;
    #pragma unroll
    for (int i = 0; i < RS; ++i) proj += a_st[i*S::nq + q]*wo.w[i]*wo.ow[i];
    S::forcing(m, e)[q] = proj*proj*2*st[(ND + 1)*S::nq + q]/st[ND*S::nq + q];
  }
}

// Flow_bc::apply_diffusion (ghost state = inside, src/Boundary_condition.cpp:43-52) or
// flux_diffusion (ghost LDG flux = -inside, :54-60) over nv face variables, at face point q of
// boundary connection i; run by k_sav_neighbor_ldg's thread for that point first.
template <int ND, int RS>
__device__ __forceinline__ void sav_bc_diffusion_point(const SavDev& m, int i, int q, int flux)
{
  using S = SavShape<ND, RS>;
  constexpr int nfq = S::nfq;
  const int* c = m.bc_con + 4*i;
  const double* in = S::slot(m, c[0], flux);
  double* gh = S::slot(m, c[1], flux);
  for (int v = 0; v < S::nv; ++v) gh[v*nfq + q] = flux ? -in[v*nfq + q] : in[v*nfq + q];
}

// Spatial<pde::Smooth_art_visc>::Neighbor (reconcile = 0: the LDG average of the three traces
// on both sides) and Neighbor_reconcile (reconcile = 1, include/Spatial.hpp:716-759).
template <int ND, int RS>
__global__ void k_sav_neighbor_ldg(SavDev m, int reconcile)
{
  using S = SavShape<ND, RS>;
  constexpr int nfq = S::nfq;
  const long total = (long)(m.n_car_con + m.n_def_con + m.n_bc_con)*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    int s0, s1, dir;
    const double* nrml = sav_connection(m, ND, nfq, int(t/nfq), s0, s1, dir);
    const int q = int(t%nfq);
    const int i_bc = int(t/nfq) - m.n_car_con - m.n_def_con;
    if (i_bc >= 0) sav_bc_diffusion_point<ND, RS>(m, i_bc, q, reconcile);   // the ghost first
    const bool deformed = nrml != nullptr;
    const int q1 = deformed ? perm_index<ND, RS>(dir, q) : q;
    double* l0 = S::slot(m, s0, true);
    double* l1 = S::slot(m, s1, true);
    if (!reconcile) {
      const double* f0 = S::slot(m, s0, false);
      const double* f1 = S::slot(m, s1, false);
      #pragma unroll
      for (int v = 0; v < S::n_sav; ++v) {
        const double avg = .5*(f0[v*nfq + q] + f1[v*nfq + q1]);
        l0[v*nfq + q] = avg;
        l1[v*nfq + q1] = avg;
      }
    } else {
      int sign0 = 1, sign1 = 1;
      if (deformed) {
        sign0 = 1 - 2*(((dir >> 4) & 1) == 0);
        sign1 = 1 - 2*(((dir >> 5) & 1) == 1);
      }
      #pragma unroll
      for (int v = 0; v < S::n_sav; ++v) {
        const double a = l0[v*nfq + q], b = l1[v*nfq + q1];
        double avg = 0;
        avg += .5*sign0*a;
        avg += .5*sign1*b;
        l0[v*nfq + q] = sign0*avg - a;
        l1[v*nfq + q1] = sign1*avg - b;
      }
    }
  }
}

// Shared memory of k_sav_local_diffusion, in doubles: the three unknowns [3][nq], the fluxes
// [nd][3][nq] (which first hold, one dimension d at a time, the metric products n_dj u_v
// [nd (j)][3][nq] of the deformed gradient), and the gradient rows' boundary corrections
// [nd][nd][3][nfq][2].
template <int ND, int RS>
struct SavDiffSmem {
  using S = SavShape<ND, RS>;
  static constexpr int rows = 0;
  static constexpr int flux = S::n_sav*S::nq;
  static constexpr int bf = flux + ND*S::n_sav*S::nq;
  static constexpr size_t bytes = sizeof(double)*(size_t)(bf + ND*ND*S::n_sav*S::nfq*2);
};

// Boundary corrections of the gradient rows of dimension d, one task per (j, unknown, row):
// fb_s - B_s.x with x the row of the unknown (times the metric normal n_dj on deformed
// elements: rows of s_x, [j][3][nq]) and fb_s its LDG face value (times the face normal).
template <int ND, int RS>
__device__ __forceinline__ void sav_diff_row_corrections(const SavDev& m, const SavTab<RS>& tab, int e, int d,
                                                         bool deformed, const double* s_x, double* s_bf)
{
  using S = SavShape<ND, RS>;
  constexpr int nfq = S::nfq, n_sav = S::n_sav, nq = S::nq;
  const int n_j = deformed ? ND : 1;
  const double* la = S::slot(m, e*2*ND + 2*d, true);
  const double* lb = S::slot(m, e*2*ND + 2*d + 1, true);
  for (int t = threadIdx.x; t < n_j*n_sav*nfq; t += blockDim.x) {
    const int i_fq = t%nfq, v = (t/nfq)%n_sav, j = t/(nfq*n_sav);
    double x[RS];
    #pragma unroll
    for (int k = 0; k < RS; ++k) x[k] = s_x[(j*n_sav + v)*nq + S::row_qpoint(d, i_fq, k)];
    double fb0 = la[v*nfq + i_fq], fb1 = lb[v*nfq + i_fq];
    if (deformed) {
      const double* fna = m.face_nrml + ((size_t)(e - m.n_car)*2*ND + 2*d)*ND*nfq;
      fb0 = fna[j*nfq + i_fq]*fb0;
      fb1 = fna[ND*nfq + j*nfq + i_fq]*fb1;
    }
    double b0 = 0., b1 = 0.;
    #pragma unroll
    for (int k = 0; k < RS; ++k) { b0 += tab.bound[k]*x[k]; b1 += tab.bound[RS + k]*x[k]; }
    const int r = ((d*ND + j)*n_sav + v)*nfq + i_fq;
    s_bf[2*r] = fb0 - b0;
    s_bf[2*r + 1] = fb1 - b1;
  }
}

// Spatial<pde::Smooth_art_visc>::Local, first stage (include/Spatial.hpp:326-509): the
// unknowns are forcing rows 1-3, their gradient (times the Jacobian determinant, product rule
// with the metric on deformed elements, Spatial.hpp:371-402) gives the flux -gradient.normal
// (diffusivity 1); the source of unknown v is f(forcing row v)/diff_time with f = |x| for rows
// 0 and 2 and sqrt|x| for row 1 (pde.hpp:422-429); the flux's face values go to the LDG faces
// and write_update adds (pde.hpp:379-387). One CTA per element, one thread per quadrature
// point. On deformed elements each point forms its metric products n_dj u_v once per
// dimension into shared memory, where the row tasks (boundary corrections) and the points'
// derivatives read them. Divisions by the element size and the Jacobian determinant are
// multiplications by reciprocals formed once: an ulp per operation from the reference's
// divisions, of which there were 36 per point, each costing about ten FP64 operations.
template <int ND, int RS>
__global__ void __launch_bounds__(SavShape<ND, RS>::block)
k_sav_local_diffusion(SavDev m, SavTab<RS> tab, double dt, double diff_time)
{
  using S = SavShape<ND, RS>;
  using L = SavDiffSmem<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, n_sav = S::n_sav;
  extern __shared__ double s_mem[];
  double* s_r = s_mem + L::rows;   // [3][nq]
  double* s_f = s_mem + L::flux;   // [ND][3][nq]; during the gradient: products [ND (j)][3][nq]
  double* s_bf = s_mem + L::bf;    // [ND (d)][ND (j)][3][nfq][2]
  const int e = blockIdx.x;
  const int q = threadIdx.x;
  const bool deformed = e >= m.n_car;
  const double* st = m.elem + (size_t)e*(S::nv + 3)*nq;
  double* fc = S::forcing(m, e);
  const double d_pos = m.nom_size[e];
  const double inv_dpos = 1./d_pos;
  const int ed = e - m.n_car;
  const double* nrml = deformed ? m.jac + (size_t)ed*(ND*ND + 1)*nq : nullptr;
  if (q < nq) {
    #pragma unroll
    for (int v = 0; v < n_sav; ++v) s_r[v*nq + q] = fc[(1 + v)*nq + q];
  }
  double g[n_sav][ND];
  #pragma unroll
  for (int v = 0; v < n_sav; ++v)
    #pragma unroll
    for (int d = 0; d < ND; ++d) g[v][d] = 0.;
  if (deformed) {
    // grad_j u_v = sum_d [D_d (n_dj u_v) + lift_d (n^f_dj u^f_v - B_d (n_dj u_v))] / size
    #pragma unroll
    for (int d = 0; d < ND; ++d) {
      __syncthreads();   // s_r staged (d = 0); the previous dimension's products read
      if (q < nq) {
        #pragma unroll
        for (int j = 0; j < ND; ++j) {
          const double n_dj = nrml[(d*ND + j)*nq + q];
          #pragma unroll
          for (int v = 0; v < n_sav; ++v) s_f[(j*n_sav + v)*nq + q] = n_dj*s_r[v*nq + q];
        }
      }
      __syncthreads();
      sav_diff_row_corrections<ND, RS>(m, tab, e, d, true, s_f, s_bf);
      __syncthreads();
      if (q < nq) {
        const int stride = ipow(RS, ND - 1 - d);
        const int i = (q/stride)%RS;
        const int i_fq = (q/(stride*RS))*stride + q%stride;
        const int r0 = q - i*stride;
        #pragma unroll
        for (int j = 0; j < ND; ++j)
          #pragma unroll
          for (int v = 0; v < n_sav; ++v) {
            double x[RS];
            #pragma unroll
            for (int k = 0; k < RS; ++k) x[k] = s_f[(j*n_sav + v)*nq + r0 + k*stride];
            const int r = ((d*ND + j)*n_sav + v)*nfq + i_fq;
            g[v][j] = accumulate_derivative_bf<RS, 1>(g[v][j], tab, x, s_bf[2*r], s_bf[2*r + 1], i);
          }
      }
    }
    #pragma unroll
    for (int v = 0; v < n_sav; ++v)
      #pragma unroll
      for (int j = 0; j < ND; ++j) g[v][j] *= inv_dpos;   // the sum over d, scaled once
    __syncthreads();   // every product read before the fluxes overwrite them
  } else {
    __syncthreads();
    #pragma unroll
    for (int d = 0; d < ND; ++d) sav_diff_row_corrections<ND, RS>(m, tab, e, d, false, s_r, s_bf);
    __syncthreads();
    if (q < nq) {
      #pragma unroll
      for (int d = 0; d < ND; ++d) {
        const int stride = ipow(RS, ND - 1 - d);
        const int i = (q/stride)%RS;
        const int i_fq = (q/(stride*RS))*stride + q%stride;
        const int r0 = q - i*stride;
        #pragma unroll
        for (int v = 0; v < n_sav; ++v) {
          double x[RS];
          #pragma unroll
          for (int k = 0; k < RS; ++k) x[k] = s_r[v*nq + r0 + k*stride];
          const int r = ((d*ND)*n_sav + v)*nfq + i_fq;   // the task layout with j = 0
          g[v][d] = accumulate_derivative_bf<RS, 1>(0., tab, x, s_bf[2*r], s_bf[2*r + 1], i)*inv_dpos;
        }
      }
    }
  }
  // flux -gradient.normal (Spatial.hpp:405-442)
  if (q < nq) {
    const double inv_det = deformed ? 1./nrml[ND*ND*nq + q] : 1.;
    #pragma unroll
    for (int v = 0; v < n_sav; ++v) {
      if (deformed) {
        #pragma unroll
        for (int d = 0; d < ND; ++d) g[v][d] *= inv_det;
      }
      #pragma unroll
      for (int i = 0; i < ND; ++i) {
        double acc = 0.;
        #pragma unroll
        for (int j = 0; j < ND; ++j) acc += -g[v][j]*(deformed ? nrml[(i*ND + j)*nq + q] : (i == j ? 1. : 0.));
        s_f[(i*n_sav + v)*nq + q] = acc;
      }
    }
  }
  __syncthreads();
  // the flux's face values to the LDG faces: one thread per (dimension, face point, unknown)
  for (int t = threadIdx.x; t < ND*nfq*n_sav; t += blockDim.x) {
    const int v = t%n_sav, i_fq = (t/n_sav)%nfq, d = t/(n_sav*nfq);
    double x[RS];
    #pragma unroll
    for (int k = 0; k < RS; ++k) x[k] = s_f[(d*n_sav + v)*nq + S::row_qpoint(d, i_fq, k)];
    #pragma unroll
    for (int s = 0; s < 2; ++s) {
      double acc = 0.;
      #pragma unroll
      for (int k = 0; k < RS; ++k) acc += tab.bound[s*RS + k]*x[k];
      S::slot(m, e*2*ND + 2*d + s, true)[v*nfq + i_fq] = acc;
    }
  }
  if (q >= nq) return;
  // source, then the interior divergence of the flux (Spatial.hpp:445-470)
  double mult_src = d_pos;
  const double det = deformed ? nrml[ND*ND*nq + q] : 1.;
  if (deformed) mult_src *= det;
  double rate[n_sav];
  #pragma unroll
  for (int v = 0; v < n_sav; ++v) {
    const double f = fabs(fc[v*nq + q]);
    rate[v] = mult_src*(((v == 1) ? sqrt(f) : f)/diff_time);
  }
  #pragma unroll
  for (int d = 0; d < ND; ++d) {
    const int stride = ipow(RS, ND - 1 - d);
    const int i = (q/stride)%RS;
    const int r0 = q - i*stride;
    #pragma unroll
    for (int v = 0; v < n_sav; ++v) {
      double acc = rate[v];   // rate -= D.flux, one FMA chain
      #pragma unroll
      for (int k = 0; k < RS; ++k) acc -= tab.diff[i*RS + k]*s_f[(d*n_sav + v)*nq + r0 + k*stride];
      rate[v] = acc;
    }
  }
  double mult = dt*st[S::nv*nq + q]/d_pos;
  if (deformed) mult /= det;
  #pragma unroll
  for (int v = 0; v < n_sav; ++v) {
    double u = 0.;
    u += rate[v];
    u *= mult;
    fc[(1 + v)*nq + q] += u;
  }
}

// Spatial<pde::Smooth_art_visc>::Reconcile_ldg_flux (include/Spatial.hpp:543-594): lift of the
// flux differences, then the critical write_update (pde.hpp:379-387): add, then divide by
// pseudo = 1 + tss cheby/diff_time. One thread per quadrature point.
template <int ND, int RS>
__global__ void k_sav_reconcile(SavDev m, SavTab<RS> tab, double dt, double diff_time, double cheby)
{
  using S = SavShape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, n_sav = S::n_sav;
  const long total = (long)m.n_elem*nq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int e = int(t/nq), q = int(t%nq);
    const bool deformed = e >= m.n_car;
    double rate[n_sav];
    #pragma unroll
    for (int v = 0; v < n_sav; ++v) rate[v] = 0.;
    #pragma unroll
    for (int d = 0; d < ND; ++d) {
      const int stride = ipow(RS, ND - 1 - d);
      const int i = (q/stride)%RS;
      const int i_fq = (q/(stride*RS))*stride + q%stride;
      const double* la = S::slot(m, e*2*ND + 2*d, true);
      const double* lb = S::slot(m, e*2*ND + 2*d + 1, true);
      #pragma unroll
      for (int v = 0; v < n_sav; ++v) {
        double l = 0.;
        l += tab.lift[i*2]*la[v*nfq + i_fq];
        l += tab.lift[i*2 + 1]*lb[v*nfq + i_fq];
        rate[v] = 1.*rate[v] + -l;
      }
    }
    const double* st = m.elem + (size_t)e*(S::nv + 3)*nq;
    const double tss = st[S::nv*nq + q];
    const double size = deformed ? m.nom_size[e]*m.jac[((size_t)(e - m.n_car)*(ND*ND + 1) + ND*ND)*nq + q]
                                 : m.nom_size[e];
    const double mult = dt*tss/size;
    const double inv_pseudo = 1/(1 + tss*cheby/diff_time);   // one division for the three unknowns
    double* fc = S::forcing(m, e);
    #pragma unroll
    for (int v = 0; v < n_sav; ++v) {
      double x = fc[(1 + v)*nq + q];
      x += rate[v]*mult;
      x *= inv_pseudo;
      fc[(1 + v)*nq + q] = x;
    }
  }
}

// Solver.cpp:552-575: the bulk AV coefficient us_max f/(us_max + f) from forcing row 3, the
// element's share of art_visc_residual (partials[e]) and the momentum put back.
template <int ND, int RS>
__global__ void k_sav_finish(SavDev m, AvTab<RS, double> wt, double mult, double us_max)
{
  using S = SavShape<ND, RS>;
  constexpr int nq = S::nq;
  __shared__ double s_sum[32];
  for (int e = blockIdx.x; e < m.n_elem; e += gridDim.x) {
    double* st = m.elem + (size_t)e*(S::nv + 3)*nq;
    double* av = st + (S::nv + 1)*nq;
    const double* fc = S::forcing(m, e);
    double volume = 1.;
    #pragma unroll
    for (int d = 0; d < ND; ++d) volume *= m.nom_size[e];
    double part = 0.;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      double qw = 1.;
      #pragma unroll
      for (int d = 0; d < ND; ++d) qw *= wt.w[(q/ipow(RS, ND - 1 - d))%RS];
      const double f = mult*fc[(S::n_forcing - 1)*nq + q];
      const double new_av = us_max*f/(us_max + f);
      const double diff = av[q] - new_av;
      part += diff*diff*qw*volume;
      av[q] = new_av;
      const double scale = sqrt(2*st[ND*nq + q]*st[(ND + 1)*nq + q]);
      #pragma unroll
      for (int d = 0; d < ND; ++d) st[d*nq + q] *= scale;
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x/32] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      double sum = 0.;
      for (int w = 0; w < (int)(blockDim.x + 31)/32; ++w) sum += s_sum[w];
      m.partials[e] = sum;
    }
    __syncthreads();
  }
}

// The advection state starts at 1 (Solver's constructor, src/Solver.cpp:201-211).
static __global__ void k_sav_init(double* aux, long n_elem, int n_aux, int first_row, int n_rows, int nq)
{
  const long total = n_elem*n_rows*nq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const long e = t/((long)n_rows*nq), k = t%((long)n_rows*nq);
    aux[(e*n_aux + first_row)*nq + k] = 1.;
  }
}

// sum of the per-element partials, then sqrt
static __global__ void k_sav_residual(const double* partials, int n, double* out)
{
  __shared__ double s_sum[256];
  double acc = 0.;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partials[i];
  s_sum[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x/2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s_sum[threadIdx.x] += s_sum[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sqrt(s_sum[0]);
}

} // namespace hx
