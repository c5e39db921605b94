// kernels.cuh -- sm_103a device code of the DG spatial operator and stage update.
//
// One CUDA thread per quadrature point (volume kernels) or per face quadrature point
// (face kernels). A CTA holds EPB whole elements; their state, fluxes and per-row
// boundary corrections are staged in shared memory so that the tensor-product line
// contractions of Derivative (include/Derivative.hpp:50-60) read each row from shared
// memory. The contractions are rs x rs with rs <= 8, far too thin for tcgen05 tensor
// cores, so they run on the FP64 (plain form) or FP32 (mixed form) pipes.
//
// Arithmetic follows the reference operation by operation (sums in ascending index
// order, same association) so that the FP64 form agrees with the CPU oracle to
// roundoff; nvcc contracts a*b + c into FMAs, which is the only systematic difference.
//
// Template parameters: ND (2, 3), RS (row size), R (compute type: double, or float in
// the mixed form), DEF (deformed elements / connections), VISC (LDG viscous path).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include "../../include/hexed_gpu.h"

namespace hx {

constexpr int ipow(int b, int e) { int r = 1; for (int i = 0; i < e; ++i) r *= b; return r; }
constexpr double heat_rat = 1.4;                 // include/pde.hpp:51
constexpr double specific_gas_air = 287.05287;   // include/constants.hpp:44

// Basis tables of one row size (generated by hexed_gb300/basis.py), passed by value as a
// kernel parameter and copied to shared memory by each CTA.
template <int RS>
struct Tab {
  double diff[RS*RS];      // diff[i*RS + j] = L_j'(x_i)
  double bound[2*RS];      // bound[s*RS + j] = L_j(s)
  double lift[RS*2];       // lift[i*2 + s] (include/Derivative.hpp:22-28)
  double filter[RS*RS];
  double node[RS];
  double weight[RS];
  double prolong[2*RS*RS];
  double restrict_[2*RS*RS];
  double ortho_last[RS];   // highest-degree orthonormal Legendre mode at the nodes
  double max_cfl, min_eig_diffusion, step_ratio;
};

// Device view of the arena (include/hexed_gpu.h). `face` is stored as FaceT.
// Device view of the arena. FaceT is the storage type of the face traces, the residual cache
// and the metric normals the flux kernels read: double in the FP64 form; float in the mixed
// form, where those arrays are FP32 copies (the FP64 metrics stay in `jac`). The FP64 form's
// stage update multiplies by the FP64 `inv_det`; the mixed form's volume kernel forms 1/det
// in float from the determinant row of its staged normals.
template <typename FaceT>
struct Dev {
  int n_car, n_def, n_elem, n_slot, n_car_con, n_def_con, n_bc_con, n_ref;
  double* elem;
  FaceT* rcache;
  FaceT* face;
  const double* nom_size;
  const double* vert_tss;
  const float* vert_tss_f;    // mixed form: the same in float (Max_dt's point scales); null in FP64
  const double* jac;          // FP64 [n_def][nd*nd + 1][nq]
  const double* inv_det;      // FP64 [n_def][nq], 1/det
  const FaceT* nrm;           // [n_def][nd*nd + 1][nq], reference-level normals in FaceT
  const FaceT* face_nrml;
  const int* car_con;
  const int* def_con;
  const FaceT* def_con_nrml;
  const int* bc_con;
  const double* bc_nrml;      // FP64 boundary normals (boundary conditions)
  const FaceT* bc_nrml_t;     // the same in FaceT (face flux)
  double* bc_cache;
  const int* ref_face;
  const hexed_bc_spec* bc_spec;
  // Mixed form: reference state of each element [n_elem][nv]; its face traces, and the
  // fluxes its kernels form, are differences from it (see RefState). Null in the FP64 form.
  const double* ref;
  const float* ref_terms;   // mixed form: RefState<ND, float> of each element
  // Mixed form: slots at or beyond elem_slot_end (boundary ghost faces, hanging-face mortars)
  // belong to no element; slot_elem[slot - elem_slot_end] is the element whose reference
  // state their traces are offsets from (the inside element, the coarse element)
  int elem_slot_end;
  const int* slot_elem;
  double* scalars;       // [0] dt of the current stage, [1] raw max_dt, ...
  double* partials;      // per-block reduction scratch
  int* status;           // device-side error flags
  // 1: the viscous chain and Max_dt compute pde::Fix_therm_admis (include/pde.hpp:437-493)
  // instead of Navier-Stokes: no convection, flux = -gradient*normal, diffusivity 1; its
  // boundary conditions copy the inside state to the ghost face and negate the inside LDG
  // flux (src/Solver.cpp:103-114, 1067-1072)
  int fta;
};

enum { SC_DT = 0, SC_MAXDT = 1, SC_FLOWTIME = 2, SC_SAVED = 4, SC_N = 8 };   // SC_SAVED: copy of [0, 2)

template <int ND, int RS>
struct Shape {
  static constexpr int nq = ipow(RS, ND);
  static constexpr int nfq = nq/RS;
  static constexpr int nv = ND + 2;
  static constexpr int nvert = 1 << ND;
  static constexpr int epb = nq >= 256 ? 1 : 256/nq;     // elements per CTA
  static constexpr int threads_raw = epb*nq;
  static constexpr int threads = (threads_raw + 31)/32*32;
  static constexpr int slot_dof = 2*nv*nfq;
  static __host__ __device__ constexpr int stride(int d) { return ipow(RS, ND - 1 - d); }
};

// Threads of a volume-kernel CTA holding EPB elements (whole warps).
template <int ND, int RS, int EPB>
struct Tile { static constexpr int threads = (EPB*ipow(RS, ND) + 31)/32*32; };
template <typename T> __device__ __forceinline__ T load(const T* p) { return __ldg(p); }

// ------------------------------------------------------------------- conversions (mixed form)
// IEEE 754 binary64 <-> binary32 conversions written with integer operations, from the
// format definitions. The hardware conversions between double and float issue on the FP64
// pipe, which on this GPU runs at a small fraction of the FP32 rate and was the busiest unit
// of the mixed-form kernels; these run on the integer pipes. f32_of rounds to nearest even
// (as __double2float_rn does) where the result is a normal float, and gives signed zero
// below the normal range (no float subnormals), +-inf above it and NaN for NaN. f64_of is
// exact for normal floats, gives signed zero for float zeros and subnormals and keeps inf
// and NaN.
__device__ __forceinline__ float f32_of(double x)
{
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned a = hi & 0x7fffffffu;   // high word of |x|
  // |x| as float bits with the mantissa cut to 23 bits: the exponent rebiased from 1023 to 127
  // (minus 896 << 20) and the 64-bit pattern shifted left by 3, keeping its high word
  unsigned t = __funnelshift_l(lo, a - 0x38000000u, 3);
  // round to nearest even on the 29 bits cut away: carry out of rest + (half - 1) + lsb; a
  // carry may reach the exponent (up to inf, as rounding should)
  t += ((lo & 0x1fffffffu) + 0x0fffffffu + (t & 1u)) >> 29;
  // outside the float normal range, 2^-126 <= |x| < 2^128 (one unsigned compare; rare)
  if (a - 0x38100000u >= 0x47f00000u - 0x38100000u)
    t = a < 0x38100000u ? 0u : (a > 0x7ff00000u || (a == 0x7ff00000u && lo)) ? 0x7fc00000u : 0x7f800000u;
  return __uint_as_float((hi & 0x80000000u) | t);
}

__device__ __forceinline__ double f64_of(float f)
{
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u, a = b & 0x7fffffffu;
  // a normal float: exponent and mantissa move together (right by 3), the exponent rebiased
  unsigned hi = sign | ((a >> 3) + 0x38000000u);
  unsigned lo = b << 29;
  if (a - 0x00800000u >= 0x7f800000u - 0x00800000u) {   // zero, subnormal, inf or NaN (rare)
    const unsigned m = b & 0x7fffffu;
    hi = a < 0x00800000u ? sign : sign | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u);
    lo = a < 0x00800000u ? 0u : lo;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// Self-check of f32_of / f64_of against the hardware conversions (__double2float_rn and
// the float-to-double widening): counts inputs whose results differ in any bit, skipping
// inputs whose float result is subnormal (f32_of flushes those to zero by design).
static __global__ void k_check_conversions(const double* in, long n, unsigned long long* mismatches)
{
  for (long i = blockIdx.x*(long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x*blockDim.x) {
    const double x = in[i];
    const float hw = __double2float_rn(x);
    const float sw = f32_of(x);
    const float ahw = fabsf(hw);
    if (ahw > 0.f && ahw < 1.17549435e-38f) continue;
    bool bad = isnan(hw) ? !isnan(sw) : __float_as_uint(hw) != __float_as_uint(sw);
    const double wide_hw = double(hw), wide_sw = f64_of(hw);
    bad = bad || (isnan(wide_hw) ? !isnan(wide_sw) : __double_as_longlong(wide_hw) != __double_as_longlong(wide_sw));
    if (bad) atomicAdd(mismatches, 1ull);
  }
}

// double -> compute type R (identity for double)
template <typename R>
__device__ __forceinline__ R to_R(double x)
{
  if constexpr (std::is_same<R, float>::value) return f32_of(x);
  else return x;
}

// ------------------------------------------------------------------- PDE pieces
// Navier_stokes<visc>::Pde::Computation (include/pde.hpp:72-175), one qpoint.
template <int ND, typename R>
struct Conv {
  // Divisions by the density are multiplications by its reciprocal (one division per
  // qpoint): the FP64 pipe of this GPU is the bound, and each double division costs
  // several FMAs. This moves results by at most an ulp per operation.
  R mass, inv_mass, kin_ener, pressure;
  __device__ __forceinline__ explicit Conv(const R* s)
  {
    mass = s[ND];
    inv_mass = R(1)/mass;
    kin_ener = 0;
    #pragma unroll
    for (int d = 0; d < ND; ++d) kin_ener += s[d]*s[d];
    kin_ener *= R(.5)*inv_mass;
    pressure = R(heat_rat - 1.)*(s[ND + 1] - kin_ener);
  }
  // compute_flux_conv for one flux direction n (pde.hpp:108-122). `p_mom` is the pressure
  // used in the momentum flux: the pressure itself, or (mixed form) its deviation from an
  // element reference pressure whose contribution is accounted for in double elsewhere.
  __device__ __forceinline__ void flux(const R* s, const R* n, R* f, R p_mom) const
  {
    R fm = 0;
    #pragma unroll
    for (int j = 0; j < ND; ++j) fm += s[j]*n[j];
    f[ND] = fm;
    R vol_flux = fm*inv_mass;
    f[ND + 1] = (s[ND + 1] + pressure)*vol_flux;
    #pragma unroll
    for (int j = 0; j < ND; ++j) f[j] = s[j]*vol_flux + p_mom*n[j];
  }
  __device__ __forceinline__ void flux(const R* s, const R* n, R* f) const { flux(s, n, f, pressure); }
};

template <int ND, typename R>
__device__ __forceinline__ R char_speed(const R* s, R inv_mass) // pde.hpp:161-166
{
  R sound_speed = sqrt(R(heat_rat*(heat_rat - 1))*s[ND + 1]*inv_mass);
  R sq = 0;
  #pragma unroll
  for (int d = 0; d < ND; ++d) sq += s[d]*s[d];
  return sound_speed + sqrt(sq)*inv_mass;
}

// Reference state of the mixed form and the parts of its flux the offset flux needs.
// Each element has its own reference (by default the mean of its initial state), so the
// offsets carry only the variation inside the element. `lo` is the rounding error of `s`: the
// double reference is s + lo to about 2^-48 relative, so the difference of two elements'
// references, (s1 - s0) + (lo1 - lo0), has the relative accuracy of float whatever the
// references' size (the face kernels convert traces between neighbouring elements with it).
template <int ND, typename R>
struct alignas(16) RefState {   // 16-byte aligned: read with vector loads (float: 3 nd + 7 values, padded)
  R s[ND + 2];   // conserved reference state
  R lo[ND + 2];  // ref - s (zero in double)
  R v[ND];       // its velocity
  R v_sq;        // |v|^2
  R h;           // E + p
  R inv_mass;    // 1/density
  __device__ __forceinline__ void set(const double* ref)
  {
    #pragma unroll
    for (int i = 0; i < ND + 2; ++i) {
      s[i] = to_R<R>(ref[i]);
      lo[i] = to_R<R>(ref[i] - double(s[i]));
    }
    const R inv = R(1)/s[ND];
    inv_mass = inv;
    v_sq = 0;
    #pragma unroll
    for (int j = 0; j < ND; ++j) { v[j] = s[j]*inv; v_sq += v[j]*v[j]; }
    h = s[ND + 1] + R(heat_rat - 1.)*(s[ND + 1] - R(.5)*s[ND]*v_sq);
  }
};

// RefState<ND, float> of every element from its double reference state
template <int ND>
__global__ void k_ref_terms(const double* ref, int n_elem, RefState<ND, float>* out)
{
  for (int e = blockIdx.x*blockDim.x + threadIdx.x; e < n_elem; e += gridDim.x*blockDim.x)
    out[e].set(ref + (size_t)e*(ND + 2));
}

// f(u).n - f(u_ref).n of the convective flux (pde.hpp:108-122) from the offset state
// d = u - u_ref, with inv_mass = 1/u[ND] of the full state u. Every term is an offset times a bounded
// factor, so in float the result carries the relative accuracy of the offsets and not of the
// full fluxes (no difference of nearly equal fluxes is formed):
//   dv = (dm - v_ref drho)/rho, dp = (gamma-1)(dE - (drho |v_ref|^2 + rho (v + v_ref).dv)/2),
//   mass dm.n, momentum dm (v.n) + m_ref (dv.n) + dp n, energy (dE + dp)(v.n) + h_ref (dv.n).
// The reference flux itself drops out of the scheme: its volume derivative and its face
// terms cancel by the discrete metric identity (free-stream preservation).
template <int ND, typename R>
__device__ __forceinline__ void flux_delta(const R* u, const R* d, const RefState<ND, R>& r, R inv_mass,
                                           const R* n, R* f)
{
  R v[ND], dv[ND];
  R dkin2 = d[ND]*r.v_sq;
  #pragma unroll
  for (int j = 0; j < ND; ++j) {
    v[j] = u[j]*inv_mass;
    dv[j] = (d[j] - r.v[j]*d[ND])*inv_mass;
    dkin2 += u[ND]*(v[j] + r.v[j])*dv[j];
  }
  const R dp = R(heat_rat - 1.)*(d[ND + 1] - R(.5)*dkin2);
  R vn = 0, dvn = 0, dmn = 0;
  #pragma unroll
  for (int j = 0; j < ND; ++j) { vn += v[j]*n[j]; dvn += dv[j]*n[j]; dmn += d[j]*n[j]; }
  #pragma unroll
  for (int i = 0; i < ND; ++i) f[i] = d[i]*vn + r.s[i]*dvn + dp*n[i];
  f[ND] = dmn;
  f[ND + 1] = (d[ND + 1] + dp)*vn + r.h*dvn;
}

// Transport_model constants folded on the host, in the compute type of the kernel
// (include/Transport_model.hpp:21-44).
template <typename R>
struct TmT {
  R const_val, ref_val, inv_sqrt_ref_temp, ref_temp_plus_offset, temp_offset;
};
template <typename R>
inline TmT<R> make_tm(const hexed_transport& t)
{
  return {R(t.const_val), R(t.ref_val), R(1./sqrt(t.ref_temp)), R(t.ref_temp + t.temp_offset), R(t.temp_offset)};
}

template <typename R>
__device__ __forceinline__ R transport_coef(const TmT<R>& t, R sqrt_temp) // Transport_model.hpp:35-38
{
  R r = sqrt_temp*R(t.inv_sqrt_ref_temp);
  R p3 = r*r*r;
  return R(t.const_val) + R(t.ref_val)*p3*R(t.ref_temp_plus_offset)/(sqrt_temp*sqrt_temp + R(t.temp_offset));
}

template <int ND, typename R>
struct DiffScalars { // compute_scalars_diff (pde.hpp:130-138)
  R bulk_av, laplacian_av, mu, energy_cond;
  __device__ __forceinline__ DiffScalars(const R* s, const Conv<ND, R>& c, R bulk, R lap,
                                         const TmT<R>& visc, const TmT<R>& cond)
  {
    bulk_av = fabs(bulk);
    laplacian_av = fabs(lap);
    R sqrt_temp = sqrt(fmax((s[ND + 1] - c.kin_ener)*c.inv_mass, R(0))*R(heat_rat - 1)*R(1./specific_gas_air));
    R k;
    if (visc.inv_sqrt_ref_temp == cond.inv_sqrt_ref_temp && visc.ref_temp_plus_offset == cond.ref_temp_plus_offset &&
        visc.temp_offset == cond.temp_offset) {
      // the two models share their temperature law (Sutherland with one offset, as for air):
      // its factor (T/T_ref)^1.5 (T_ref + S)/(T + S) once, with one division
      const R r = sqrt_temp*R(visc.inv_sqrt_ref_temp);
      const R law = r*r*r*R(visc.ref_temp_plus_offset)/(sqrt_temp*sqrt_temp + R(visc.temp_offset));
      mu = R(visc.const_val) + R(visc.ref_val)*law;
      k = R(cond.const_val) + R(cond.ref_val)*law;
    } else {
      mu = transport_coef(visc, sqrt_temp);
      k = transport_coef(cond, sqrt_temp);
    }
    energy_cond = k*R(heat_rat - 1)*R(1./specific_gas_air);
  }
};

// compute_flux_diff (pde.hpp:142-158): g[v][j] gradient, nrm[j][i] (physical j, reference i)
template <int ND, typename R, bool IDENT>
__device__ __forceinline__ void flux_diff(const R* s, const Conv<ND, R>& c, const DiffScalars<ND, R>& df,
                                          const R (&g)[ND + 2][ND], const R (&nrm)[ND][ND], R (&out)[ND + 2][ND])
{
  const R mass = c.mass, inv_mass = c.inv_mass;
  R veloc[ND];
  #pragma unroll
  for (int i = 0; i < ND; ++i) veloc[i] = s[i]*inv_mass;
  R vg[ND][ND];
  #pragma unroll
  for (int i = 0; i < ND; ++i)
    #pragma unroll
    for (int j = 0; j < ND; ++j) vg[i][j] = (g[i][j] - veloc[i]*g[ND][j])*inv_mass;
  R trace = 0;
  #pragma unroll
  for (int i = 0; i < ND; ++i) trace += vg[i][i];
  const R bulk_term = (df.bulk_av*mass - R(2./3.)*df.mu)*trace;
  R stress[ND][ND];
  #pragma unroll
  for (int i = 0; i < ND; ++i)
    #pragma unroll
    for (int j = 0; j < ND; ++j) stress[i][j] = df.mu*(vg[i][j] + vg[j][i]) + (i == j ? bulk_term : R(0));
  R fd[ND + 2][ND];
  #pragma unroll
  for (int v = 0; v < ND + 2; ++v)
    #pragma unroll
    for (int j = 0; j < ND; ++j) fd[v][j] = -df.laplacian_av*g[v][j];
  #pragma unroll
  for (int i = 0; i < ND; ++i)
    #pragma unroll
    for (int j = 0; j < ND; ++j) fd[i][j] -= stress[i][j];
  const R coef = -s[ND + 1]*inv_mass*inv_mass;
  #pragma unroll
  for (int j = 0; j < ND; ++j) {
    R vvg = 0;
    #pragma unroll
    for (int i = 0; i < ND; ++i) vvg += veloc[i]*vg[i][j];
    R ieg = coef*g[ND][j] + g[ND + 1][j]*inv_mass - vvg;
    R vs = 0;
    #pragma unroll
    for (int i = 0; i < ND; ++i) vs += veloc[i]*stress[i][j];
    fd[ND + 1][j] -= vs + df.energy_cond*ieg;
  }
  #pragma unroll
  for (int v = 0; v < ND + 2; ++v) {
    #pragma unroll
    for (int i = 0; i < ND; ++i) {
      if (IDENT) { out[v][i] = fd[v][i]; continue; }
      R acc = 0;
      #pragma unroll
      for (int j = 0; j < ND; ++j) acc += fd[v][j]*nrm[j][i];
      out[v][i] = acc;
    }
  }
}

// Fix_therm_admis::compute_flux_diff (include/pde.hpp:481-485): flux = -gradient*normal
template <int ND, typename R, bool IDENT>
__device__ __forceinline__ void flux_fta(const R (&g)[ND + 2][ND], const R (&nrm)[ND][ND], R (&out)[ND + 2][ND])
{
  #pragma unroll
  for (int v = 0; v < ND + 2; ++v) {
    #pragma unroll
    for (int i = 0; i < ND; ++i) {
      if (IDENT) { out[v][i] = -g[v][i]; continue; }
      R acc = 0;
      #pragma unroll
      for (int j = 0; j < ND; ++j) acc += -g[v][j]*nrm[j][i];
      out[v][i] = acc;
    }
  }
}

// Face-1 index that lands at face-0 qpoint q after Face_permutation::match_faces
// (transpose then flip; include/Spatial.hpp:85-129, include/Kernel_connection.hpp:55-85).
template <int ND, int RS>
__device__ __forceinline__ int perm_index(int dir, int q)
{
  const int i_dim0 = dir & 3, i_dim1 = (dir >> 2) & 3;
  const bool s0 = (dir >> 4) & 1, s1 = (dir >> 5) & 1;
  const bool flip_n0 = !s0, flip_n1 = s1;
  const bool flip_tan = (i_dim0 != i_dim1) && (flip_n0 == flip_n1);
  const bool transpose = ((i_dim0 == 0) && (i_dim1 == 2)) || ((i_dim0 == 2) && (i_dim1 == 0));
  if constexpr (ND == 3) {
    int r = q%RS, c = q/RS;
    if (flip_tan) {
      const bool colwise = (i_dim0 > 3 - i_dim0 - i_dim1) != transpose;
      if (colwise) r = RS - 1 - r; else c = RS - 1 - c;
    }
    int idx = r + c*RS;
    if (transpose) idx = (idx%RS)*RS + idx/RS;
    return idx;
  } else {
    return flip_tan ? RS - 1 - q : q;
  }
}

__device__ __forceinline__ int bc_dir(int packed) // {{d,d},{ifs,!ifs}} (include/connection.hpp:378)
{
  int d = packed & 3, ifs = (packed >> 2) & 1;
  return d | (d << 2) | (ifs << 4) | ((!ifs) << 5);
}

// Per-CTA shared copy of the 1-D operators in the compute type.
template <int RS, typename R>
struct STab {
  R diff[RS*RS];
  R bound[2*RS];
  R lift[2*RS];
  R filter[RS*RS];
  __device__ __forceinline__ void load(const Tab<RS>& t)
  {
    for (int i = threadIdx.x; i < RS*RS; i += blockDim.x) { diff[i] = R(t.diff[i]); filter[i] = R(t.filter[i]); }
    for (int i = threadIdx.x; i < 2*RS; i += blockDim.x) { bound[i] = R(t.bound[i]); lift[i] = R(t.lift[i]); }
  }
};

// ------------------------------------------------------------------- row tasks
// The tensor-product line contractions of Derivative (include/Derivative.hpp:50-60) run as
// row tasks: one thread per (element, variable, row along a dimension). A task loads the RS
// values of its row from shared memory once, forms both boundary products B.x from them and
// writes all RS outputs of the row. The 1-D operators are kernel parameters indexed only by
// compile-time constants, so each entry is a constant operand of its FMA. Per output this is
// one shared-memory load and one store, where a thread per point loads the whole row and the
// operator row for every output.
template <int RS, typename R>
struct RowTab {
  R diff[RS*RS];     // diff[i*RS + j] = L_j'(x_i)
  R bound[2*RS];     // bound[s*RS + j] = L_j(s)
  R lift[2*RS];      // lift[i*2 + s] (include/Derivative.hpp:22-28)
  R filter[RS*RS];
};

template <int RS, typename R>
inline RowTab<RS, R> make_rowtab(const Tab<RS>& t)
{
  RowTab<RS, R> r;
  for (int i = 0; i < RS*RS; ++i) { r.diff[i] = R(t.diff[i]); r.filter[i] = R(t.filter[i]); }
  for (int i = 0; i < 2*RS; ++i) { r.bound[i] = R(t.bound[i]); r.lift[i] = R(t.lift[i]); }
  return r;
}

// Element-local index of the first point of row r (0 <= r < nfq) along dimension D.
template <int ND, int RS, int D>
__device__ __forceinline__ int row_base(int r)
{
  constexpr int stride = Shape<ND, RS>::stride(D);
  return (r/stride)*stride*RS + r%stride;
}

template <int RS, int STRIDE, typename R>
__device__ __forceinline__ void load_row(const R* p, R (&x)[RS])
{
  #pragma unroll
  for (int k = 0; k < RS; ++k) x[k] = p[k*STRIDE];
}

// a0 = B_0.x, a1 = B_1.x (the row extrapolated to its two faces)
template <int RS, typename R>
__device__ __forceinline__ void bound_dot(const RowTab<RS, R>& t, const R (&x)[RS], R& a0, R& a1)
{
  a0 = 0;
  a1 = 0;
  #pragma unroll
  for (int k = 0; k < RS; ++k) { a0 += t.bound[k]*x[k]; a1 += t.bound[RS + k]*x[k]; }
}

// (D.x)_i + lift_i.(b0, b1): Derivative::operator() at node i, with b_s the face value minus
// the extrapolated row (include/Derivative.hpp:56-60). One FMA chain, lift terms first, as in
// the FP64 body: the sums need not follow the reference's order (they agree with it to
// roundoff, far inside the parity bars), and a chain saves the separate additions.
template <int RS, typename R>
__device__ __forceinline__ R row_deriv(const RowTab<RS, R>& t, const R (&x)[RS], int i, R b0, R b1)
{
  R acc = t.lift[i*2]*b0;
  acc += t.lift[i*2 + 1]*b1;
  #pragma unroll
  for (int k = 0; k < RS; ++k) acc += t.diff[i*RS + k]*x[k];
  return acc;
}

// Calls f(std::integral_constant<int, I>()) for I = 0 .. N-1 in order.
template <int N, int I = 0, typename F>
__device__ __forceinline__ void static_for(F&& f)
{
  if constexpr (I < N) {
    f(std::integral_constant<int, I>());
    static_for<N, I + 1>(f);
  }
}

// Calls f(std::integral_constant<int, d>) for a runtime dimension d, so that a task loop
// balanced over all dimensions still sees compile-time strides.
template <int ND, typename F>
__device__ __forceinline__ void dim_switch(int d, F&& f)
{
  if (d == 0) f(std::integral_constant<int, 0>());
  else if constexpr (ND == 3) {
    if (d == 1) f(std::integral_constant<int, 1>());
    else f(std::integral_constant<int, 2>());
  } else f(std::integral_constant<int, ND - 1>());
}

// ------------------------------------------------------------------- Write_face helper
// Extrapolate an element's state (shared memory, [nv][nq]) to its 2nd face slots
// (Spatial::Write_face, include/Spatial.hpp:41-57). Called by all threads of the CTA.
template <int ND, int RS, typename R, typename FaceT, int EPB = Shape<ND, RS>::epb>
__device__ __forceinline__ void write_faces_from_smem(const Dev<FaceT>& m, const RowTab<RS, R>& rt, const R* s_u,
                                                      int e0, int e_end)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  constexpr int per_d = EPB*nv*nfq;
  // callers launch Tile<ND, RS, EPB>::threads threads (k_local, k_reconcile_ldg): a constant
  // stride, and 32-bit offsets from the CTA's first element's face slots
  constexpr int kThreads = Tile<ND, RS, EPB>::threads;
  FaceT* const face_cta = m.face + (size_t)e0*2*ND*S::slot_dof;
  for (int t = threadIdx.x; t < ND*per_d; t += kThreads) {
    const int d = t/per_d, rem = t - d*per_d;
    const int r = rem%nfq, rest = rem/nfq;
    const int v = rest%nv, le = rest/nv;
    const int e = e0 + le;
    if (EPB > 1 && e >= e_end) continue;
    dim_switch<ND>(d, [&](auto dc) {
      constexpr int D = decltype(dc)::value;
      R x[RS];
      load_row<RS, S::stride(D)>(s_u + (le*nv + v)*nq + row_base<ND, RS, D>(r), x);
      R a0, a1;
      bound_dot(rt, x, a0, a1);
      FaceT* f0 = face_cta + (le*2*ND + 2*D)*S::slot_dof + v*nfq + r;
      f0[0] = FaceT(a0);
      f0[S::slot_dof] = FaceT(a1);   // slot of face 2d + 1
    });
  }
}

// Write_face of the per-point body: the same extrapolation with the boundary rows read from
// the CTA's shared table and runtime row strides (fewer registers than the compile-time-stride
// row tasks, which the FP64 kernels' occupancy needs).
template <int ND, int RS, typename R, typename FaceT, int EPB = Shape<ND, RS>::epb>
__device__ __forceinline__ void write_faces_points(const Dev<FaceT>& m, const STab<RS, R>& st,
                                                      const R* s_u, int e0, int e_end)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  constexpr int n_task = EPB*ND*nv*nfq;
  for (int task = threadIdx.x; task < n_task; task += blockDim.x) {
    int r = task%nfq;
    int rest = task/nfq;
    int v = rest%nv; rest /= nv;
    int d = rest%ND;
    int le = rest/ND;
    int e = e0 + le;
    if (e >= e_end) continue;
    const int stride = S::stride(d);
    const int base = (r/stride)*stride*RS + r%stride;
    const R* row = s_u + (le*nv + v)*nq + base;
    R a0 = 0, a1 = 0;
    #pragma unroll
    for (int i = 0; i < RS; ++i) {
      R x = row[i*stride];
      a0 += st.bound[i]*x;
      a1 += st.bound[RS + i]*x;
    }
    FaceT* f0 = m.face + (size_t)(e*2*ND + 2*d)*S::slot_dof + v*nfq + r;
    f0[0] = FaceT(a0);
    f0[S::slot_dof] = FaceT(a1);   // slot of face 2d + 1
  }
}

// ------------------------------------------------------------------- bulk async copies
// One-dimensional bulk copy (TMA) of `bytes` contiguous bytes from global to shared memory,
// completing on an mbarrier, and the bounded wait for it. Both addresses and `bytes` must be
// multiples of 16 (the caller checks and otherwise reads global memory directly).
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
  const unsigned mb = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(mb), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gmem_src, unsigned bytes,
                                          unsigned long long* bar)
{
  const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_dst);
  const unsigned mb = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(mb), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(dst), "l"(gmem_src), "r"(bytes), "r"(mb) : "memory");
}

// Waits for phase `phase` of the mbarrier, giving up after `max_polls` polls (false).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned phase, unsigned max_polls)
{
  const unsigned mb = (unsigned)__cvta_generic_to_shared(bar);
  for (unsigned i = 0; i < max_polls; ++i) {
    unsigned done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(mb), "r"(phase) : "memory");
    if (done) return true;
  }
  return false;
}
constexpr unsigned bulk_wait_polls = 1u << 20;

// Bulk prefetch of [p, p + bytes) from HBM into L2 (no data returned to the SM); skipped unless
// the range starts on 16 bytes and its length is a multiple of 16, as the bulk copy requires.
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes)
{
  if (((reinterpret_cast<unsigned long long>(p) | bytes) & 15u) || bytes == 0) return;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"((unsigned)bytes) : "memory");
}

// The per-element arrays a volume-kernel CTA reads after its state, prefetched into L2 at its
// start so that the later per-point and per-row loads hit L2 rather than HBM: the element face
// slots, the residual cache (read by the second stage) and, for deformed elements, the metric
// normals, the determinant reciprocals and (viscous) the face normals.
template <int ND, int RS, bool DEF, bool VISC, typename FaceT>
__device__ __forceinline__ void prefetch_element_arrays(const Dev<FaceT>& m, int e0, int n_here, int stage)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  prefetch_l2(m.face + (size_t)e0*2*ND*S::slot_dof, sizeof(FaceT)*(size_t)n_here*2*ND*S::slot_dof);
  if (stage) prefetch_l2(m.rcache + (size_t)e0*nv*nq, sizeof(FaceT)*(size_t)n_here*nv*nq);
  if constexpr (DEF) {
    const size_t ed0 = (size_t)(e0 - m.n_car);
    prefetch_l2(m.nrm + ed0*(ND*ND + 1)*nq, sizeof(FaceT)*(size_t)n_here*(ND*ND + 1)*nq);
    // the float form takes the determinant from the staged normals' last row instead
    if constexpr (std::is_same<FaceT, double>::value) prefetch_l2(m.inv_det + ed0*nq, sizeof(double)*(size_t)n_here*nq);
    if constexpr (VISC) prefetch_l2(m.face_nrml + ed0*2*ND*ND*nfq, sizeof(FaceT)*(size_t)n_here*2*ND*ND*nfq);
  }
}
// status[1] bits (read by hexed_gpu_device_flags): a bulk-copy wait gave up and the kernel
// read global memory instead
constexpr int flag_bulk_wait = 1;

// ------------------------------------------------------------------- Local
// Spatial::Local (include/Spatial.hpp:326-509) fused with the stage update and Write_face.
template <int ND, int RS, typename R, bool DEF, bool VISC, int EPB = Shape<ND, RS>::epb>
struct LocalSmemPoints {
  using S = Shape<ND, RS>;
  static constexpr int per_elem = S::nv*S::nq            // s_u
                                + ND*S::nv*S::nq         // s_f
                                + (VISC ? ND*S::nv*S::nq : 0)   // s_g
                                + ND*2*S::nv*S::nfq;     // s_bf
  // [tables][mbarrier, 16 B][element states, EPB x (nv + 3) x nq doubles][s_u s_f s_g s_bf]
  static constexpr size_t tab_bytes = (sizeof(STab<RS, R>) + 15)/16*16;
  static constexpr size_t state_bytes = sizeof(double)*(size_t)EPB*(S::nv + 3)*S::nq;
  static constexpr size_t work_offset = tab_bytes + 16 + (state_bytes + 15)/16*16;
  static constexpr size_t bytes = work_offset + sizeof(R)*(size_t)per_elem*EPB + 16;
};

template <int ND, int RS, typename R, bool DEF, bool VISC, int EPB = Shape<ND, RS>::epb>
struct LocalSmemRows {
  using S = Shape<ND, RS>;
  // work fields per element, in R:
  //   s_u  [nv][nq]     offset state (Cartesian gradient, Write_face); the convective residual
  //   s_x  [ND][nv][nq] metric-weighted offset state of the deformed gradient; then the fluxes
  //   s_g  [ND][nv][nq] gradient; then the viscous fluxes (viscous path)
  //   s_vr [nv][nq]     viscous residual (viscous path)
  static constexpr int per_elem = S::nv*S::nq + ND*S::nv*S::nq + (VISC ? (ND + 1)*S::nv*S::nq : 0);
  // [mbarrier, 16 B][1/element size, EPB x R][element states, EPB x (nv + 3) x nq doubles]
  // [deformed: metric normals and determinant, EPB x (nd^2 + 1) x nq in R][work]
  // [each element's reference state and its derived terms (RefState), EPB of them]
  static constexpr size_t idp_offset = 16;
  static constexpr size_t ref_offset = idp_offset + (sizeof(R)*EPB + 15)/16*16;
  static constexpr size_t state_offset = ref_offset + (sizeof(RefState<ND, R>)*EPB + 15)/16*16;
  static constexpr size_t state_bytes = sizeof(double)*(size_t)EPB*(S::nv + 3)*S::nq;
  static constexpr size_t nrm_offset = state_offset + (state_bytes + 15)/16*16;
  static constexpr size_t nrm_bytes = DEF ? sizeof(R)*(size_t)EPB*(ND*ND + 1)*S::nq : 0;
  // [inviscid: residual cache, EPB x nv x nq in R (read by the second stage)]
  static constexpr size_t rc_offset = nrm_offset + (nrm_bytes + 15)/16*16;
  static constexpr size_t rc_bytes = VISC ? 0 : sizeof(R)*(size_t)EPB*S::nv*S::nq;
  static constexpr size_t work_offset = rc_offset + (rc_bytes + 15)/16*16;
  static constexpr size_t bytes = work_offset + sizeof(R)*(size_t)per_elem*EPB;
};

// Max_dt of one quadrature point (include/Spatial.hpp:793-826): the local time step from the
// vertex time-step scales interpolated to the point at reference coordinates `coord`, the
// characteristic speed and, for diffusion, the diffusivity. inv_cfl_c = 1/(max_cfl*conv
// safety) and inv_cfl_d = 1/(-2/min_eig_diffusion*diff safety) come from the host. Shared by
// k_max_dt and the fused local-time path of k_local.
template <int ND, int RS, typename R, bool VISC, typename FaceT>
__device__ __forceinline__ R point_step(const Dev<FaceT>& m, int e, int q, const R (&coord)[ND], R inv_cfl_c,
                                        R inv_cfl_d, const TmT<R>& visc, const TmT<R>& cond)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nv = S::nv, nvert = S::nvert;
  const double* state = m.elem + (size_t)e*(nv + 3)*nq;
  R vals[nvert];
  #pragma unroll
  for (int i = 0; i < nvert; ++i) {
    if constexpr (std::is_same<R, double>::value) vals[i] = m.vert_tss[(size_t)e*nvert + i];
    else vals[i] = m.vert_tss_f[(size_t)e*nvert + i];   // converted once per vertex, not per point
  }
  int stride = nvert;
  #pragma unroll
  for (int d = 0; d < ND; ++d) {
    stride /= 2;
    #pragma unroll
    for (int i = 0; i < (nvert >> (d + 1)); ++i) vals[i] += coord[d]*(vals[i + stride] - vals[i]);
  }
  const R spacing = vals[0];
  R s[nv];
  #pragma unroll
  for (int v = 0; v < nv; ++v) s[v] = to_R<R>(state[v*nq + q]);
  // 1/(c icc/h + nu icd/h^2) = h^2/(c icc h + nu icd): one division instead of two (each
  // costs several FP64 operations on this GPU's FP64 pipe)
  if (m.fta) return spacing*spacing/inv_cfl_d;   // Fix_therm_admis: diffusivity 1
  Conv<ND, R> c(s);
  R denom = char_speed<ND, R>(s, c.inv_mass)*inv_cfl_c*spacing;
  if constexpr (VISC) {
    DiffScalars<ND, R> df(s, c, to_R<R>(state[(nv + 1)*nq + q]), to_R<R>(state[(nv + 2)*nq + q]), visc, cond);
    R diffusivity = fabs(df.laplacian_av) + fmax(fabs(df.bulk_av) + df.mu*c.inv_mass, df.energy_cond*c.inv_mass);
    denom += diffusivity*inv_cfl_d;
  }
  return spacing*spacing/denom;
}

// Reference coordinates of point q from a node table (RS entries in R)
template <int ND, int RS, typename R, typename NodeT>
__device__ __forceinline__ void point_coords(const NodeT* node, int q, R (&coord)[ND])
{
  #pragma unroll
  for (int d = 0; d < ND; ++d) coord[d] = to_R<R>(node[(q/ipow(RS, ND - 1 - d))%RS]);
}

// Time step of a k_local launch. mode 0: the step is scalars[SC_DT] and the time-step scale
// row of the state holds each point's scale (written by k_max_dt). mode 1 (first stage of an
// update with local time stepping): the step is `dt` and the kernel computes each point's
// scale itself (point_step, as k_max_dt would) and stores it. mode 2: the step is `dt`, the
// scale row is read.
struct LocalDt {
  int mode;
  double inv_cfl_c, inv_cfl_d;   // mode 1: point_step's safety-scaled CFL reciprocals
  double dt;
};


// Offset form of the state used for face traces and derivatives: the mixed form subtracts the
// element's reference state (in double, before narrowing), so the FP32 values carry the
// variation and not the large mean; the FP64 form keeps the state as it is.
template <int ND, typename R, typename FaceT>
__device__ __forceinline__ R offset_var(const Dev<FaceT>& m, int e, int v, double x)
{
  if constexpr (std::is_same<FaceT, double>::value) return R(x);
  else return to_R<R>(x - m.ref[(size_t)e*(ND + 2) + v]);
}

// Spatial::Local (include/Spatial.hpp:326-509) with one thread per quadrature point for the
// point work and the contractions alike: each thread forms its own point's D.f + lift.(fb - B.f)
// from its row in shared memory, after per-row boundary corrections fb - B.f have been formed
// once per row.
template <int ND, int RS, typename R, bool DEF, bool VISC, typename FaceT, int EPB>
__device__ __forceinline__ void local_body_points(Dev<FaceT> m, const Tab<RS>& tab, int e_begin, int e_end, int stage,
                                           int compute_residual, int use_filter, const TmT<R>& visc,
                                           const TmT<R>& cond, const LocalDt& ldt)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  // Mixed form: traces and convective fluxes are offsets from the element's reference state
  // (flux_delta). The reference flux's parts of interior and face fluxes cancel by the discrete
  // metric identity sum_d [D.n_d + lift.(n_face - B.n_d)] = 0 (free-stream preservation), so
  // this is the same scheme up to roundoff, without differences of nearly equal floats.
  constexpr bool split = !std::is_same<FaceT, double>::value;
  using L = LocalSmemPoints<ND, RS, R, DEF, VISC, EPB>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  STab<RS, R>& st = *reinterpret_cast<STab<RS, R>*>(smem_raw);
  unsigned long long* s_bar = reinterpret_cast<unsigned long long*>(smem_raw + L::tab_bytes);
  double* s_state = reinterpret_cast<double*>(smem_raw + L::tab_bytes + 16);
  R* s_u = reinterpret_cast<R*>(smem_raw + L::work_offset);
  R* s_f = s_u + EPB*nv*nq;
  R* s_g = s_f + EPB*ND*nv*nq;
  R* s_bf = s_g + (VISC ? EPB*ND*nv*nq : 0);
  const int le = threadIdx.x/nq;
  const int q = threadIdx.x%nq;
  const int e0 = e_begin + blockIdx.x*EPB;
  const int e = e0 + le;
  const bool active = threadIdx.x < EPB*nq && e < e_end;
  // The CTA's element states ([n][nv + 3][nq], contiguous) arrive in shared memory by one bulk
  // copy while the tables load; where the range is not 16-byte aligned, threads read global
  // memory directly (same values).
  const double* g_state = m.elem + (size_t)e0*(nv + 3)*nq;
  const unsigned state_bytes = unsigned(min(EPB, e_end - e0)*(nv + 3)*nq*sizeof(double));
  const bool bulk = ((reinterpret_cast<unsigned long long>(g_state) | state_bytes) & 15u) == 0;
  if (bulk && threadIdx.x == 0) mbar_init(s_bar, 1);
  __syncthreads();
  if (bulk && threadIdx.x == 0) bulk_load(s_state, g_state, state_bytes, s_bar);
  if (threadIdx.x == 32) prefetch_element_arrays<ND, RS, DEF, VISC>(m, e0, min(EPB, e_end - e0), stage);
  st.load(tab);
  const int ed = e - m.n_car;
  const double d_pos = active ? m.nom_size[e] : 1.;
  const double inv_dpos = 1./d_pos;
  const R inv_dpos_r = split ? R(1)/to_R<R>(d_pos) : R(inv_dpos);
  const bool staged = bulk && mbar_wait(s_bar, 0, bulk_wait_polls);
  if (bulk && !staged) atomicOr(m.status + 1, flag_bulk_wait);
  const double* state_g = (staged ? s_state : g_state) + (size_t)le*(nv + 3)*nq;

  R u[nv + 2];   // state + bulk AV + Laplacian AV (include/pde.hpp:79-84)
  R up[nv];      // offset form of the state
  const double* ref_e = split ? m.ref + (size_t)(active ? e : 0)*nv : nullptr;
  R nrm[ND][ND]; // nrm[j][i] = comp.normal(j, i)
  #pragma unroll
  for (int i = 0; i < ND; ++i)
    #pragma unroll
    for (int j = 0; j < ND; ++j) nrm[j][i] = (i == j) ? R(1) : R(0);
  if (active) {
    #pragma unroll
    for (int v = 0; v < nv; ++v) {
      const double x = state_g[v*nq + q];
      up[v] = offset_var<ND, R>(m, e, v, x);
      if constexpr (split) u[v] = to_R<R>(ref_e[v]) + up[v];
      else u[v] = R(x);
    }
    u[nv] = to_R<R>(state_g[(nv + 1)*nq + q]);
    u[nv + 1] = to_R<R>(state_g[(nv + 2)*nq + q]);
    if constexpr (DEF) {
      const FaceT* nr = m.nrm + (size_t)ed*(ND*ND + 1)*nq;
      #pragma unroll
      for (int i = 0; i < ND; ++i)
        #pragma unroll
        for (int j = 0; j < ND; ++j) nrm[j][i] = R(nr[(i*ND + j)*nq + q]);
    }
  } else {
    #pragma unroll
    for (int v = 0; v < nv + 2; ++v) u[v] = R(1);
    #pragma unroll
    for (int v = 0; v < nv; ++v) up[v] = R(0);
  }
  R* my_u = s_u + le*nv*nq;
  R* my_f = s_f + le*ND*nv*nq;
  R* my_g = s_g + le*ND*nv*nq;
  R* my_bf = s_bf + le*ND*2*nv*nfq;
  // position of this qpoint in its row along each dimension
  int node_of[ND], base_of[ND], row_of[ND];
  #pragma unroll
  for (int d = 0; d < ND; ++d) {
    const int stride = S::stride(d);
    node_of[d] = (q/stride)%RS;
    base_of[d] = q - node_of[d]*stride;
    row_of[d] = (q/(stride*RS))*stride + q%stride;
  }

  R grad[nv][ND];
  if constexpr (VISC) {
    // ---- gradient times Jacobian determinant (Spatial.hpp:371-402)
    #pragma unroll
    for (int v = 0; v < nv; ++v)
      #pragma unroll
      for (int j = 0; j < ND; ++j) grad[v][j] = 0;
    if constexpr (!DEF) {
      if (threadIdx.x < EPB*nq) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) my_u[v*nq + q] = up[v];
      }
      __syncthreads();
      // per-row boundary corrections: bf_s = face_state_s - B_s . row
      constexpr int n_task = EPB*ND*nv*nfq;
      for (int task = threadIdx.x; task < n_task; task += blockDim.x) {
        int r = task%nfq, rest = task/nfq;
        int v = rest%nv; rest /= nv;
        int d = rest%ND; int l = rest/ND;
        int ee = e0 + l;
        if (ee >= e_end) continue;
        const int stride = S::stride(d);
        const R* row = s_u + (l*nv + v)*nq + (r/stride)*stride*RS + r%stride;
        R a0 = 0, a1 = 0;
        #pragma unroll
        for (int i = 0; i < RS; ++i) { R x = row[i*stride]; a0 += st.bound[i]*x; a1 += st.bound[RS + i]*x; }
        const FaceT* fl = m.face + (size_t)(ee*2*ND + 2*d)*S::slot_dof + nv*nfq + v*nfq + r;
        R* bf = s_bf + ((l*ND + d)*2*nv)*nfq;
        bf[v*nfq + r] = R(fl[0]) - a0;
        bf[(nv + v)*nfq + r] = R(fl[S::slot_dof]) - a1;
      }
      __syncthreads();
      if (active) {
        #pragma unroll
        for (int d = 0; d < ND; ++d) {
          const int stride = S::stride(d);
          const int i = node_of[d];
          const R* bf = my_bf + d*2*nv*nfq;
          #pragma unroll
          for (int v = 0; v < nv; ++v) {
            // one FMA chain per output, lift terms first (as in row_deriv)
            const R* row = my_u + v*nq + base_of[d];
            R acc = st.lift[i*2]*bf[v*nfq + row_of[d]];
            acc += st.lift[i*2 + 1]*bf[(nv + v)*nfq + row_of[d]];
            #pragma unroll
            for (int j = 0; j < RS; ++j) acc += st.diff[i*RS + j]*row[j*stride];
            grad[v][d] = acc*inv_dpos_r;
          }
        }
      }
    } else {
      const FaceT* nr = m.nrm + (size_t)ed*(ND*ND + 1)*nq;
      #pragma unroll 1
      for (int d = 0; d < ND; ++d) {
        __syncthreads(); // previous use of s_f / s_bf finished
        if (active) {
          #pragma unroll
          for (int j = 0; j < ND; ++j) {
            R nd_ = R(nr[(d*ND + j)*nq + q]);
            #pragma unroll
            for (int v = 0; v < nv; ++v) my_f[(j*nv + v)*nq + q] = nd_*up[v];
          }
        }
        __syncthreads();
        constexpr int n_task = EPB*ND*nv*nfq;
        const int stride = S::stride(d);
        for (int task = threadIdx.x; task < n_task; task += blockDim.x) {
          int r = task%nfq, rest = task/nfq;
          int v = rest%nv; rest /= nv;
          int j = rest%ND; int l = rest/ND;
          int ee = e0 + l;
          if (ee >= e_end) continue;
          const int eed = ee - m.n_car;
          const R* row = s_f + ((l*ND + j)*nv + v)*nq + (r/stride)*stride*RS + r%stride;
          R a0 = 0, a1 = 0;
          #pragma unroll
          for (int i = 0; i < RS; ++i) { R x = row[i*stride]; a0 += st.bound[i]*x; a1 += st.bound[RS + i]*x; }
          const FaceT* fl = m.face + (size_t)(ee*2*ND + 2*d)*S::slot_dof + nv*nfq + v*nfq + r;
          const FaceT* fnr = m.face_nrml + ((size_t)eed*2*ND + 2*d)*ND*nfq + j*nfq + r;
          R b0 = R(fnr[0])*R(fl[0]);
          R b1 = R(fnr[ND*nfq])*R(fl[S::slot_dof]);
          R* bf = s_bf + ((l*ND + j)*2*nv)*nfq;
          bf[v*nfq + r] = b0 - a0;
          bf[(nv + v)*nfq + r] = b1 - a1;
        }
        __syncthreads();
        if (active) {
          const int i = node_of[d];
          #pragma unroll
          for (int j = 0; j < ND; ++j) {
            const R* bf = my_bf + j*2*nv*nfq;
            #pragma unroll
            for (int v = 0; v < nv; ++v) {
              // the sum over d accumulates unscaled in one FMA chain per output, lift terms
              // first; the 1/size factor is applied once after the last dimension
              const R* row = my_f + (j*nv + v)*nq + base_of[d];
              R acc = grad[v][j];
              acc += st.lift[i*2]*bf[v*nfq + row_of[d]];
              acc += st.lift[i*2 + 1]*bf[(nv + v)*nfq + row_of[d]];
              #pragma unroll
              for (int jj = 0; jj < RS; ++jj) acc += st.diff[i*RS + jj]*row[jj*stride];
              grad[v][j] = acc;
            }
          }
        }
      }
      #pragma unroll
      for (int v = 0; v < nv; ++v)
        #pragma unroll
        for (int j = 0; j < ND; ++j) grad[v][j] *= inv_dpos_r;
    }
    __syncthreads(); // s_f / s_bf are reused below
  }

  // ---- fluxes (Spatial.hpp:405-442)
  if (active) {
    Conv<ND, R> c(u);
    RefState<ND, R> rs;   // formed here, not kept live through the gradient part
    if constexpr (split) rs.set(ref_e);
    #pragma unroll
    for (int i = 0; i < ND; ++i) {
      R col[ND], f[nv];
      #pragma unroll
      for (int j = 0; j < ND; ++j) col[j] = nrm[j][i];
      if (VISC && m.fta) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) f[v] = R(0);   // Fix_therm_admis has no convection
      } else if constexpr (split) flux_delta<ND, R>(u, up, rs, c.inv_mass, col, f);
      else c.flux(u, col, f);
      #pragma unroll
      for (int v = 0; v < nv; ++v) my_f[(i*nv + v)*nq + q] = f[v];
    }
    if constexpr (VISC) {
      R g[nv][ND];
      const R inv_det = DEF ? to_R<R>(m.inv_det[(size_t)ed*nq + q]) : R(1);
      #pragma unroll
      for (int v = 0; v < nv; ++v)
        #pragma unroll
        for (int j = 0; j < ND; ++j) g[v][j] = DEF ? grad[v][j]*inv_det : grad[v][j];
      R fd[nv][ND];
      if (m.fta) {
        flux_fta<ND, R, !DEF>(g, nrm, fd);
      } else {
        DiffScalars<ND, R> df(u, c, u[nv], u[nv + 1], visc, cond);
        flux_diff<ND, R, !DEF>(u, c, df, g, nrm, fd);
      }
      #pragma unroll
      for (int i = 0; i < ND; ++i)
        #pragma unroll
        for (int v = 0; v < nv; ++v) my_g[(i*nv + v)*nq + q] = fd[v][i];
    }
  }
  __syncthreads();

  // ---- per-row boundary corrections of the convective flux; viscous flux to LDG faces
  {
    constexpr int n_task = EPB*ND*nv*nfq;
    for (int task = threadIdx.x; task < n_task; task += blockDim.x) {
      int r = task%nfq, rest = task/nfq;
      int v = rest%nv; rest /= nv;
      int d = rest%ND; int l = rest/ND;
      int ee = e0 + l;
      if (ee >= e_end) continue;
      const int stride = S::stride(d);
      const int off = (r/stride)*stride*RS + r%stride;
      const R* row = s_f + ((l*ND + d)*nv + v)*nq + off;
      R a0 = 0, a1 = 0;
      #pragma unroll
      for (int i = 0; i < RS; ++i) { R x = row[i*stride]; a0 += st.bound[i]*x; a1 += st.bound[RS + i]*x; }
      FaceT* fl = m.face + (size_t)(ee*2*ND + 2*d)*S::slot_dof + v*nfq + r;
      R* bf = s_bf + ((l*ND + d)*2*nv)*nfq;
      // Fix_therm_admis: no convective flux, in the faces as in the volume
      const bool conv = !(VISC && m.fta);
      bf[v*nfq + r] = (conv ? R(fl[0]) : R(0)) - a0;
      bf[(nv + v)*nfq + r] = (conv ? R(fl[S::slot_dof]) : R(0)) - a1;
      if constexpr (VISC) {
        const R* rg = s_g + ((l*ND + d)*nv + v)*nq + off;
        R g0 = 0, g1 = 0;
        #pragma unroll
        for (int i = 0; i < RS; ++i) { R x = rg[i*stride]; g0 += st.bound[i]*x; g1 += st.bound[RS + i]*x; }
        fl[nv*nfq] = FaceT(g0);
        fl[S::slot_dof + nv*nfq] = FaceT(g1);
      }
    }
  }
  __syncthreads();

  // ---- residual (Spatial.hpp:445-470)
  R rate[nv], vrate[nv];
  #pragma unroll
  for (int v = 0; v < nv; ++v) { rate[v] = 0; vrate[v] = 0; }
  if (active) {
    #pragma unroll
    for (int d = 0; d < ND; ++d) {
      const int stride = S::stride(d);
      const int i = node_of[d];
      const R* bf = my_bf + d*2*nv*nfq;
      #pragma unroll
      for (int v = 0; v < nv; ++v) {
        // rate -= D.f + lift.(f* - B.f) as one FMA chain per output over all dimensions
        const R* row = my_f + (d*nv + v)*nq + base_of[d];
        R acc = rate[v];
        acc -= st.lift[i*2]*bf[v*nfq + row_of[d]];
        acc -= st.lift[i*2 + 1]*bf[(nv + v)*nfq + row_of[d]];
        #pragma unroll
        for (int j = 0; j < RS; ++j) acc -= st.diff[i*RS + j]*row[j*stride];
        rate[v] = acc;
        if constexpr (VISC) {
          const R* rg = my_g + (d*nv + v)*nq + base_of[d];
          R ag = vrate[v];
          #pragma unroll
          for (int j = 0; j < RS; ++j) ag -= st.diff[i*RS + j]*rg[j*stride];
          vrate[v] = ag;
        }
      }
    }
  }

  // ---- modal filter (Spatial.hpp:473-481), one dimension at a time through shared memory
  if (use_filter) {
    #pragma unroll 1
    for (int d = 0; d < ND; ++d) {
      __syncthreads();
      if (active) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) { my_f[v*nq + q] = rate[v]; my_f[(nv + v)*nq + q] = vrate[v]; }
      }
      __syncthreads();
      if (active) {
        const int stride = S::stride(d);
        const int i = node_of[d];
        #pragma unroll
        for (int v = 0; v < 2*nv; ++v) {
          const R* row = my_f + v*nq + base_of[d];
          R acc = 0;
          #pragma unroll
          for (int j = 0; j < RS; ++j) acc += st.filter[i*RS + j]*row[j*stride];
          if (v < nv) rate[v] = acc; else vrate[v - nv] = acc;
        }
      }
    }
  }

  // ---- stage update (Spatial.hpp:484-503): the state accumulates in double
  if (active) {
    const double dt = ldt.mode ? ldt.dt : m.scalars[SC_DT];
    const double update_coef = stage ? dt*tab.step_ratio : dt;
    double* st_w = m.elem + (size_t)e*(nv + 3)*nq;
    FaceT* rc = m.rcache + (size_t)e*nv*nq;
    double tss;
    if (ldt.mode == 1) {
      R coord[ND];
      point_coords<ND, RS>(tab.node, q, coord);
      const R step = point_step<ND, RS, R, VISC>(m, e, q, coord, to_R<R>(ldt.inv_cfl_c), to_R<R>(ldt.inv_cfl_d),
                                                 visc, cond);
      if constexpr (split) tss = f64_of(step);
      else tss = step;
      st_w[nv*nq + q] = tss;
    } else {
      tss = state_g[nv*nq + q];
    }
    if constexpr (!split) {
      double mult = update_coef*tss*inv_dpos;
      if constexpr (DEF) mult *= m.inv_det[(size_t)ed*nq + q];
      #pragma unroll
      for (int v = 0; v < nv; ++v) {
        double uu = double(rate[v]);
        if (stage) {
          uu -= rc[v*nq + q];
        } else {
          if (!(VISC && m.fta)) rc[v*nq + q] = uu;   // Fix_therm_admis keeps no residual cache
          if constexpr (VISC) uu += double(vrate[v]);
        }
        uu *= mult;
        if (compute_residual) rc[v*nq + q] = FaceT(uu);
        else {
          double nu = state_g[v*nq + q] + uu;
          st_w[v*nq + q] = nu;
          up[v] = offset_var<ND, R>(m, e, v, nu);
        }
      }
    } else {
      // Mixed form: the increment is formed in float; only its accumulation into the state
      // is a double add. The offset-form trace of the new state is the old one plus the
      // increment.
      R mult = to_R<R>(update_coef)*to_R<R>(tss)*inv_dpos_r;
      if constexpr (DEF) mult *= to_R<R>(m.inv_det[(size_t)ed*nq + q]);
      #pragma unroll
      for (int v = 0; v < nv; ++v) {
        R ur = rate[v];
        if (stage) {
          ur -= R(rc[v*nq + q]);
        } else {
          if (!(VISC && m.fta)) rc[v*nq + q] = FaceT(ur);
          if constexpr (VISC) ur += vrate[v];
        }
        const R inc = ur*mult;
        if (compute_residual) rc[v*nq + q] = FaceT(inc);
        else {
          st_w[v*nq + q] = state_g[v*nq + q] + f64_of(inc);
          up[v] += inc;
        }
      }
    }
  }
  // ---- Write_face of the new state (Spatial.hpp:507); the viscous path defers it
  if constexpr (!VISC) {
    __syncthreads();
    if (active) {
      #pragma unroll
      for (int v = 0; v < nv; ++v) my_u[v*nq + q] = up[v];
    }
    __syncthreads();
    write_faces_points<ND, RS, R, FaceT, EPB>(m, st, s_u, e0, e_end);
  }
  // a bulk copy whose wait gave up must still land before the CTA's shared memory is released
  if (bulk && !staged) mbar_wait(s_bar, 0, bulk_wait_polls);
}

// Spatial::Local (include/Spatial.hpp:326-509). Point work (state, fluxes, stage update) runs
// one thread per quadrature point; the line contractions run as row tasks over the CTA's
// shared-memory fields. Every output is Derivative's, each contraction one FMA chain
// (row_deriv).
template <int ND, int RS, typename R, bool DEF, bool VISC, typename FaceT, int EPB>
__device__ __forceinline__ void local_body_rows(Dev<FaceT> m, const Tab<RS>& tab, const RowTab<RS, R>& rt,
                                                int e_begin, int e_end, int stage, int compute_residual, int use_filter,
                                                const TmT<R>& visc, const TmT<R>& cond, const LocalDt& ldt)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  // the CTA size k_local is launched with (its launch bound): task loops stride by a constant,
  // so one whose tasks fit in a CTA compiles to a single guarded pass
  constexpr int kThreads = Tile<ND, RS, EPB>::threads;
  // Mixed form: traces and convective fluxes are offsets from the element's reference state
  // (flux_delta). The reference flux's parts of interior and face fluxes cancel by the discrete
  // metric identity sum_d [D.n_d + lift.(n_face - B.n_d)] = 0 (free-stream preservation), so
  // this is the same scheme up to roundoff, without differences of nearly equal floats.
  constexpr bool split = !std::is_same<FaceT, double>::value;
  using L = LocalSmemRows<ND, RS, R, DEF, VISC, EPB>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* s_bar = reinterpret_cast<unsigned long long*>(smem_raw);
  R* s_idp = reinterpret_cast<R*>(smem_raw + L::idp_offset);
  RefState<ND, R>* s_ref = reinterpret_cast<RefState<ND, R>*>(smem_raw + L::ref_offset);
  double* s_state = reinterpret_cast<double*>(smem_raw + L::state_offset);
  R* s_n = reinterpret_cast<R*>(smem_raw + L::nrm_offset);   // deformed: [EPB][nd^2 + 1][nq]
  R* s_u = reinterpret_cast<R*>(smem_raw + L::work_offset);
  R* s_x = s_u + EPB*nv*nq;
  R* s_g = s_x + EPB*ND*nv*nq;
  R* s_vr = s_g + (VISC ? EPB*ND*nv*nq : 0);
  static_assert(sizeof(FaceT) == sizeof(R), "the row-task body stages FaceT metric normals as R");
  const int le = threadIdx.x/nq;
  const int q = threadIdx.x%nq;
  const int e0 = e_begin + blockIdx.x*EPB;
  // the CTA's first element's face slots and (deformed) face normals: row tasks address their
  // element's rows from these with 32-bit offsets
  FaceT* const face_cta = m.face + (size_t)e0*2*ND*S::slot_dof;
  const FaceT* const fnrml_cta = DEF ? m.face_nrml + (size_t)(e0 - m.n_car)*2*ND*ND*nfq : nullptr;
  const int e = e0 + le;
  const bool active = threadIdx.x < EPB*nq && e < e_end;
  const int n_here = min(EPB, e_end - e0);
  // The CTA's element states ([n][nv + 3][nq], contiguous) and, for deformed elements, their
  // metric normals ([n][nd^2 + 1][nq], contiguous) arrive in shared memory by bulk copies;
  // where a range is not 16-byte aligned, threads read global memory instead (same values).
  const double* g_state = m.elem + (size_t)e0*(nv + 3)*nq;
  const unsigned state_bytes = unsigned(n_here*(nv + 3)*nq*sizeof(double));
  const bool bulk = ((reinterpret_cast<unsigned long long>(g_state) | state_bytes) & 15u) == 0;
  const FaceT* g_nrm = DEF ? m.nrm + (size_t)(e0 - m.n_car)*(ND*ND + 1)*nq : nullptr;
  const unsigned nrm_bytes = DEF ? unsigned(n_here*(ND*ND + 1)*nq*sizeof(FaceT)) : 0u;
  const bool bulk_n = DEF && bulk && ((reinterpret_cast<unsigned long long>(g_nrm) | nrm_bytes) & 15u) == 0;
  // the second stage's residual cache of inviscid elements ([n][nv][nq], contiguous)
  R* s_rc = reinterpret_cast<R*>(smem_raw + L::rc_offset);
  const FaceT* g_rc = m.rcache + (size_t)e0*nv*nq;
  const unsigned rc_bytes = unsigned(n_here*nv*nq*sizeof(FaceT));
  const bool bulk_rc = !VISC && stage && !compute_residual && bulk &&
                       ((reinterpret_cast<unsigned long long>(g_rc) | rc_bytes) & 15u) == 0;
  if (bulk && threadIdx.x == 0) mbar_init(s_bar, 1 + bulk_n + bulk_rc);
  if (threadIdx.x < EPB) {
    const int ee = e0 + threadIdx.x;
    const double dp = ee < e_end ? m.nom_size[ee] : 1.;
    s_idp[threadIdx.x] = split ? R(1)/to_R<R>(dp) : R(1./dp);
    // the element's reference state in the compute type, formed once instead of per point
    if constexpr (split) if (ee < e_end) s_ref[threadIdx.x] = reinterpret_cast<const RefState<ND, R>*>(m.ref_terms)[ee];
  }
  __syncthreads();
  if (bulk && threadIdx.x == 0) {
    bulk_load(s_state, g_state, state_bytes, s_bar);
    if (bulk_n) bulk_load(s_n, g_nrm, nrm_bytes, s_bar);
    if (bulk_rc) bulk_load(s_rc, g_rc, rc_bytes, s_bar);
  }
  if (threadIdx.x == 32) prefetch_element_arrays<ND, RS, DEF, VISC>(m, e0, n_here, stage);
  const int ed = e - m.n_car;
  const double d_pos = active ? m.nom_size[e] : 1.;
  const double inv_dpos = 1./d_pos;
  const R inv_dpos_r = split ? R(1)/to_R<R>(d_pos) : R(inv_dpos);
  const bool staged = bulk && mbar_wait(s_bar, 0, bulk_wait_polls);
  if (bulk && !staged) atomicOr(m.status + 1, flag_bulk_wait);
  const double* state_g = (staged ? s_state : g_state) + (size_t)le*(nv + 3)*nq;
  if constexpr (DEF) {
    // normals not staged by the bulk copy: each point copies its own (visible after the next
    // barrier, before any other thread reads them)
    if (!(bulk_n && staged) && active) {
      const FaceT* nr = m.nrm + (size_t)ed*(ND*ND + 1)*nq;
      #pragma unroll
      for (int k = 0; k <= ND*ND; ++k) s_n[(le*(ND*ND + 1) + k)*nq + q] = R(nr[k*nq + q]);   // normals, determinant
    }
  }
  // comp.normal(j, i) of this thread's point, in shared memory (deformed elements)
  auto normal = [&](int l, int j, int i, int p) { return s_n[(l*(ND*ND + 1) + i*ND + j)*nq + p]; };

  R u[nv + 2];   // state + bulk AV + Laplacian AV (include/pde.hpp:79-84)
  R up[nv];      // offset form of the state
  if (active) {
    #pragma unroll
    for (int v = 0; v < nv; ++v) {
      const double x = state_g[v*nq + q];
      up[v] = offset_var<ND, R>(m, e, v, x);
      if constexpr (split) u[v] = s_ref[le].s[v] + up[v];
      else u[v] = R(x);
    }
    u[nv] = to_R<R>(state_g[(nv + 1)*nq + q]);
    u[nv + 1] = to_R<R>(state_g[(nv + 2)*nq + q]);
  } else {
    #pragma unroll
    for (int v = 0; v < nv + 2; ++v) u[v] = R(1);
    #pragma unroll
    for (int v = 0; v < nv; ++v) up[v] = R(0);
  }

  R grad[nv][ND];
  if constexpr (VISC) {
    // ---- gradient times Jacobian determinant (Spatial.hpp:371-402)
    if constexpr (!DEF) {
      if (active) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) s_u[(le*nv + v)*nq + q] = up[v];
      }
      __syncthreads();
      // grad[v][d] along each row: D.u + lift.(face LDG state - B.u), over 1/size
      constexpr int per_d = EPB*nv*nfq;
      for (int t = threadIdx.x; t < ND*per_d; t += kThreads) {
        const int d = t/per_d, rem = t - d*per_d;
        const int r = rem%nfq, rest = rem/nfq;
        const int v = rest%nv, l = rest/nv;
        const int ee = e0 + l;
        if (EPB > 1 && ee >= e_end) continue;   // one element per CTA: always in range
        dim_switch<ND>(d, [&](auto dc) {
          constexpr int D = decltype(dc)::value;
          constexpr int stride = S::stride(D);
          const int base = row_base<ND, RS, D>(r);
          R x[RS];
          load_row<RS, stride>(s_u + (l*nv + v)*nq + base, x);
          R a0, a1;
          bound_dot(rt, x, a0, a1);
          const FaceT* fl = face_cta + (l*2*ND + 2*D)*S::slot_dof + nv*nfq + v*nfq + r;
          const R b0 = R(fl[0]) - a0, b1 = R(fl[S::slot_dof]) - a1;
          const R idp = s_idp[l];
          R* g = s_g + ((l*ND + D)*nv + v)*nq + base;
          #pragma unroll
          for (int i = 0; i < RS; ++i) g[i*stride] = row_deriv(rt, x, i, b0, b1)*idp;
        });
      }
    } else {
      // grad[v][j] = sum_d [D_d.(n_dj u) + lift_d.(n_face u_face - B_d.(n_dj u))] / size. One task
      // per (variable, row) forms all nd products n_dj u along its row from the staged offset
      // state and normals, sharing the row's state and face values.
      if (active) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) s_u[(le*nv + v)*nq + q] = up[v];
      }
      static_for<ND>([&](auto dc) {
        constexpr int d = decltype(dc)::value;
        __syncthreads();   // d = 0: s_u and s_n complete; d > 0: the previous dimension's tasks are done
        constexpr int stride = S::stride(d);
        constexpr int n_task = EPB*nv*nfq;
        for (int t = threadIdx.x; t < n_task; t += kThreads) {
          const int r = t%nfq, rest = t/nfq;
          const int v = rest%nv, l = rest/nv;
          const int ee = e0 + l;
          if (EPB > 1 && ee >= e_end) continue;   // one element per CTA: always in range
          const int base = row_base<ND, RS, d>(r);
          R xu[RS];
          load_row<RS, stride>(s_u + (l*nv + v)*nq + base, xu);
          const FaceT* fl = face_cta + (l*2*ND + 2*d)*S::slot_dof + nv*nfq + v*nfq + r;
          const R fl0 = R(fl[0]), fl1 = R(fl[S::slot_dof]);
          const FaceT* fnr = fnrml_cta + (l*2*ND + 2*d)*ND*nfq + r;
          const R idp = s_idp[l];
          #pragma unroll
          for (int j = 0; j < ND; ++j) {
            const R* nrow = s_n + (l*(ND*ND + 1) + d*ND + j)*nq + base;
            R x[RS];
            #pragma unroll
            for (int k = 0; k < RS; ++k) x[k] = nrow[k*stride]*xu[k];
            R a0, a1;
            bound_dot(rt, x, a0, a1);
            const R b0 = R(fnr[j*nfq])*fl0 - a0;
            const R b1 = R(fnr[ND*nfq + j*nfq])*fl1 - a1;
            R* g = s_g + ((l*ND + j)*nv + v)*nq + base;
            #pragma unroll
            for (int i = 0; i < RS; ++i) {
              const R o = row_deriv(rt, x, i, b0, b1);
              g[i*stride] = d ? g[i*stride] + o*idp : o*idp;
            }
          }
        }
      });
    }
    __syncthreads();
    if (active) {
      #pragma unroll
      for (int v = 0; v < nv; ++v)
        #pragma unroll
        for (int j = 0; j < ND; ++j) grad[v][j] = s_g[((le*ND + j)*nv + v)*nq + q];
    }
  }

  // ---- fluxes (Spatial.hpp:405-442): s_x [i][v] convective, s_g [i][v] viscous (each point
  // overwrites only its own gradient entries)
  if (active) {
    Conv<ND, R> c(u);
    RefState<ND, R> rs;   // read here, not kept live through the gradient part
    if constexpr (split) rs = s_ref[le];
    R nrm[ND][ND]; // nrm[j][i] = comp.normal(j, i)
    #pragma unroll
    for (int i = 0; i < ND; ++i)
      #pragma unroll
      for (int j = 0; j < ND; ++j) nrm[j][i] = DEF ? normal(le, j, i, q) : (i == j) ? R(1) : R(0);
    #pragma unroll
    for (int i = 0; i < ND; ++i) {
      R col[ND], f[nv];
      #pragma unroll
      for (int j = 0; j < ND; ++j) col[j] = nrm[j][i];
      if (VISC && m.fta) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) f[v] = R(0);   // Fix_therm_admis has no convection
      } else if constexpr (split) flux_delta<ND, R>(u, up, rs, c.inv_mass, col, f);
      else c.flux(u, col, f);
      #pragma unroll
      for (int v = 0; v < nv; ++v) s_x[((le*ND + i)*nv + v)*nq + q] = f[v];
    }
    if constexpr (VISC) {
      R g[nv][ND];
      // 1/det from the staged normals' determinant row (float; no double array read)
      const R inv_det = DEF ? R(1)/s_n[(le*(ND*ND + 1) + ND*ND)*nq + q] : R(1);
      #pragma unroll
      for (int v = 0; v < nv; ++v)
        #pragma unroll
        for (int j = 0; j < ND; ++j) g[v][j] = DEF ? grad[v][j]*inv_det : grad[v][j];
      R fd[nv][ND];
      if (m.fta) {
        flux_fta<ND, R, !DEF>(g, nrm, fd);
      } else {
        DiffScalars<ND, R> df(u, c, u[nv], u[nv + 1], visc, cond);
        flux_diff<ND, R, !DEF>(u, c, df, g, nrm, fd);
      }
      #pragma unroll
      for (int i = 0; i < ND; ++i)
        #pragma unroll
        for (int v = 0; v < nv; ++v) s_g[((le*ND + i)*nv + v)*nq + q] = fd[v][i];
    }
  }

  // ---- residual (Spatial.hpp:445-470), one dimension at a time: s_u += -(D.f + lift.(f* - B.f));
  // viscous: s_vr += -D.g, and B.g to the faces' LDG slots
  static_for<ND>([&](auto dc) {
    constexpr int d = decltype(dc)::value;
    __syncthreads();
    constexpr int stride = S::stride(d);
    constexpr int n_task = EPB*nv*nfq;
    for (int t = threadIdx.x; t < n_task; t += kThreads) {
      const int r = t%nfq, rest = t/nfq;
      const int v = rest%nv, l = rest/nv;
      const int ee = e0 + l;
      if (EPB > 1 && ee >= e_end) continue;   // one element per CTA: always in range
      const int base = row_base<ND, RS, d>(r);
      R x[RS];
      load_row<RS, stride>(s_x + ((l*ND + d)*nv + v)*nq + base, x);
      R a0, a1;
      bound_dot(rt, x, a0, a1);
      FaceT* fl = face_cta + (l*2*ND + 2*d)*S::slot_dof + v*nfq + r;
      // Fix_therm_admis: no convective flux, in the faces as in the volume
      const bool conv = !(VISC && m.fta);
      const R b0 = (conv ? R(fl[0]) : R(0)) - a0, b1 = (conv ? R(fl[S::slot_dof]) : R(0)) - a1;
      R* ra = s_u + (l*nv + v)*nq + base;
      #pragma unroll
      for (int i = 0; i < RS; ++i) {
        const R o = row_deriv(rt, x, i, b0, b1);
        ra[i*stride] = d ? ra[i*stride] + -o : -o;
      }
      if constexpr (VISC) {
        load_row<RS, stride>(s_g + ((l*ND + d)*nv + v)*nq + base, x);
        bound_dot(rt, x, a0, a1);
        fl[nv*nfq] = FaceT(a0);
        fl[S::slot_dof + nv*nfq] = FaceT(a1);
        R* vr = s_vr + (l*nv + v)*nq + base;
        #pragma unroll
        for (int i = 0; i < RS; ++i) {
          R ag = 0;
          #pragma unroll
          for (int k = 0; k < RS; ++k) ag += rt.diff[i*RS + k]*x[k];
          vr[i*stride] = d ? vr[i*stride] + -ag : -ag;
        }
      }
    }
  });
  __syncthreads();
  R rate[nv], vrate[nv];
  #pragma unroll
  for (int v = 0; v < nv; ++v) { rate[v] = 0; vrate[v] = 0; }
  if (active) {
    #pragma unroll
    for (int v = 0; v < nv; ++v) {
      rate[v] = s_u[(le*nv + v)*nq + q];
      if constexpr (VISC) vrate[v] = s_vr[(le*nv + v)*nq + q];
    }
  }

  // ---- modal filter (Spatial.hpp:473-481), one dimension at a time, rows filtered in place
  if (use_filter) {
    constexpr int nf = VISC ? 2*nv : nv;   // rate, then vrate (s_x holds ND*nv >= 2*nv fields)
    static_for<ND>([&](auto dc) {
      constexpr int d = decltype(dc)::value;
      __syncthreads();
      if (active) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) {
          s_x[(le*nf + v)*nq + q] = rate[v];
          if constexpr (VISC) s_x[(le*nf + nv + v)*nq + q] = vrate[v];
        }
      }
      __syncthreads();
      constexpr int stride = S::stride(d);
      for (int t = threadIdx.x; t < EPB*nf*nfq; t += kThreads) {
        const int r = t%nfq, rest = t/nfq;
        const int v = rest%nf, l = rest/nf;
        R* row = s_x + (l*nf + v)*nq + row_base<ND, RS, d>(r);
        R x[RS];
        load_row<RS, stride>(row, x);
        #pragma unroll
        for (int i = 0; i < RS; ++i) {
          R acc = 0;
          #pragma unroll
          for (int k = 0; k < RS; ++k) acc += rt.filter[i*RS + k]*x[k];
          row[i*stride] = acc;
        }
      }
      __syncthreads();
      if (active) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) {
          rate[v] = s_x[(le*nf + v)*nq + q];
          if constexpr (VISC) vrate[v] = s_x[(le*nf + nv + v)*nq + q];
        }
      }
    });
  }

  // ---- stage update (Spatial.hpp:484-503): the state accumulates in double
  if (active) {
    const double dt = ldt.mode ? ldt.dt : m.scalars[SC_DT];
    const double update_coef = stage ? dt*tab.step_ratio : dt;
    double* st_w = m.elem + (size_t)e*(nv + 3)*nq;
    FaceT* rc = m.rcache + (size_t)e*nv*nq;
    double tss;
    if (ldt.mode == 1) {
      R coord[ND];
      point_coords<ND, RS>(tab.node, q, coord);
      const R step = point_step<ND, RS, R, VISC>(m, e, q, coord, to_R<R>(ldt.inv_cfl_c), to_R<R>(ldt.inv_cfl_d),
                                                 visc, cond);
      if constexpr (split) tss = f64_of(step);
      else tss = step;
      st_w[nv*nq + q] = tss;
    } else {
      tss = state_g[nv*nq + q];
    }
    if constexpr (!split) {
      double mult = update_coef*tss*inv_dpos;
      if constexpr (DEF) mult *= m.inv_det[(size_t)ed*nq + q];
      #pragma unroll
      for (int v = 0; v < nv; ++v) {
        double uu = double(rate[v]);
        if (stage) {
          uu -= rc[v*nq + q];
        } else {
          if (!(VISC && m.fta)) rc[v*nq + q] = uu;   // Fix_therm_admis keeps no residual cache
          if constexpr (VISC) uu += double(vrate[v]);
        }
        uu *= mult;
        if (compute_residual) rc[v*nq + q] = FaceT(uu);
        else {
          double nu = state_g[v*nq + q] + uu;
          st_w[v*nq + q] = nu;
          up[v] = offset_var<ND, R>(m, e, v, nu);
        }
      }
    } else {
      // Mixed form: the increment is formed in float; only its accumulation into the state
      // is a double add. The offset-form trace of the new state is the old one plus the
      // increment.
      R mult = to_R<R>(update_coef)*to_R<R>(tss)*inv_dpos_r;
      if constexpr (DEF) mult *= R(1)/s_n[(le*(ND*ND + 1) + ND*ND)*nq + q];
      #pragma unroll
      for (int v = 0; v < nv; ++v) {
        R ur = rate[v];
        if (stage) {
          ur -= (bulk_rc && staged) ? s_rc[(le*nv + v)*nq + q] : R(rc[v*nq + q]);
        } else {
          if (!(VISC && m.fta)) rc[v*nq + q] = FaceT(ur);
          if constexpr (VISC) ur += vrate[v];
        }
        const R inc = ur*mult;
        if (compute_residual) rc[v*nq + q] = FaceT(inc);
        else {
          st_w[v*nq + q] = state_g[v*nq + q] + f64_of(inc);
          up[v] += inc;
        }
      }
    }
  }
  // ---- Write_face of the new state (Spatial.hpp:507); the viscous path defers it
  if constexpr (!VISC) {
    __syncthreads();
    if (active) {
      #pragma unroll
      for (int v = 0; v < nv; ++v) s_u[(le*nv + v)*nq + q] = up[v];
    }
    __syncthreads();
    write_faces_from_smem<ND, RS, R, FaceT, EPB>(m, rt, s_u, e0, e_end);
  }
  // a bulk copy whose wait gave up must still land before the CTA's shared memory is released
  if (bulk && !staged) mbar_wait(s_bar, 0, bulk_wait_polls);
}

// Shared memory of one k_local CTA: the per-point body (FP64) or the row-task body (float).
template <int ND, int RS, typename R, bool DEF, bool VISC, int EPB = Shape<ND, RS>::epb>
using LocalSmem = typename std::conditional<std::is_same<R, double>::value, LocalSmemPoints<ND, RS, R, DEF, VISC, EPB>,
                                            LocalSmemRows<ND, RS, R, DEF, VISC, EPB>>::type;

// Spatial::Local (include/Spatial.hpp:293-510), one thread per quadrature point and EPB
// elements per CTA. The FP64 form uses the per-point contractions (local_body_points) and the
// float form the row tasks (local_body_rows): on this GPU the FP64 kernels are bound by the
// FP64 pipe, which the row tasks do not relieve (they ran 9-14% slower there), while the float
// kernels are bound by shared-memory instruction issue, which the row tasks cut (1.6x faster
// for the deformed viscous kernel at row size 6). MINB > 1 caps the registers for MINB
// resident CTAs per SM.
template <int ND, int RS, typename R, bool DEF, bool VISC, typename FaceT, int EPB = Shape<ND, RS>::epb, int MINB = 1>
__global__ void __launch_bounds__(Tile<ND, RS, EPB>::threads, MINB)
k_local(Dev<FaceT> m, Tab<RS> tab, RowTab<RS, R> rt, int e_begin, int e_end, int stage, int compute_residual,
        int use_filter, TmT<R> visc, TmT<R> cond, LocalDt ldt)
{
  if constexpr (std::is_same<R, double>::value)
    local_body_points<ND, RS, R, DEF, VISC, FaceT, EPB>(m, tab, e_begin, e_end, stage, compute_residual, use_filter,
                                                        visc, cond, ldt);
  else
    local_body_rows<ND, RS, R, DEF, VISC, FaceT, EPB>(m, tab, rt, e_begin, e_end, stage, compute_residual, use_filter,
                                                      visc, cond, ldt);
}

// ------------------------------------------------------------------- Reconcile_ldg_flux
// include/Spatial.hpp:543-594, fused with Write_face.
template <int ND, int RS, typename R, bool DEF>
struct ReconcileSmem {
  using S = Shape<ND, RS>;
  static constexpr size_t bytes = sizeof(STab<RS, R>) + sizeof(R)*(size_t)(S::epb*2*S::nv*S::nq) + 16;
};

template <int ND, int RS, typename R, bool DEF, typename FaceT>
__global__ void __launch_bounds__(Shape<ND, RS>::threads)
k_reconcile_ldg(Dev<FaceT> m, Tab<RS> tab, RowTab<RS, R> rt, int e_begin, int e_end, int compute_residual,
                int use_filter)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv, EPB = S::epb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  STab<RS, R>& st = *reinterpret_cast<STab<RS, R>*>(smem_raw);
  R* s_u = reinterpret_cast<R*>(smem_raw + (sizeof(STab<RS, R>) + 15)/16*16);
  R* s_t = s_u + EPB*nv*nq;
  const int le = threadIdx.x/nq, q = threadIdx.x%nq;
  const int e0 = e_begin + blockIdx.x*EPB, e = e0 + le;
  const bool active = threadIdx.x < EPB*nq && e < e_end;
  st.load(tab);
  __syncthreads();
  R tr[nv];
  #pragma unroll
  for (int v = 0; v < nv; ++v) tr[v] = 0;
  if (active) {
    #pragma unroll
    for (int d = 0; d < ND; ++d) {
      const int stride = S::stride(d);
      const int i = (q/stride)%RS;
      const int r = (q/(stride*RS))*stride + q%stride;
      const FaceT* fl = m.face + (size_t)(e*2*ND + 2*d)*S::slot_dof + nv*nfq + r;
      #pragma unroll
      for (int v = 0; v < nv; ++v) {
        R b0 = R(fl[v*nfq]), b1 = R(fl[S::slot_dof + v*nfq]);
        R acc = tr[v];   // tr -= lift.(b0, b1), one FMA chain
        acc -= st.lift[i*2]*b0;
        acc -= st.lift[i*2 + 1]*b1;
        tr[v] = acc;
      }
    }
  }
  if (use_filter) {
    R* my_t = s_t + le*nv*nq;
    #pragma unroll 1
    for (int d = 0; d < ND; ++d) {
      __syncthreads();
      if (active) {
        #pragma unroll
        for (int v = 0; v < nv; ++v) my_t[v*nq + q] = tr[v];
      }
      __syncthreads();
      if (active) {
        // the node and row start of this thread's point along d, formed here: arrays of them
        // indexed by this loop's d would sit in local memory
        const int stride = S::stride(d);
        const int i = (q/stride)%RS;
        const int base = q - i*stride;
        #pragma unroll
        for (int v = 0; v < nv; ++v) {
          const R* row = my_t + v*nq + base;
          R acc = 0;
          #pragma unroll
          for (int j = 0; j < RS; ++j) acc += st.filter[i*RS + j]*row[j*stride];
          tr[v] = acc;
        }
      }
    }
  }
  R* my_u = s_u + le*nv*nq;
  if (active) {
    const double dt = m.scalars[SC_DT];
    double* st_w = m.elem + (size_t)e*(nv + 3)*nq;
    if constexpr (std::is_same<FaceT, double>::value) {
      double mult = dt*st_w[nv*nq + q]*(1./m.nom_size[e]);
      if constexpr (DEF) mult *= m.inv_det[(size_t)(e - m.n_car)*nq + q];
      if (compute_residual) {
        FaceT* rc = m.rcache + (size_t)e*nv*nq;
        #pragma unroll
        for (int v = 0; v < nv; ++v) rc[v*nq + q] = FaceT(double(rc[v*nq + q]) + double(tr[v])*mult);
      } else {
        #pragma unroll
        for (int v = 0; v < nv; ++v) st_w[v*nq + q] += double(tr[v])*mult;
      }
    } else {
      // mixed form: increment in float, accumulated into the double state (see k_local)
      R mult = to_R<R>(dt)*to_R<R>(st_w[nv*nq + q])*(R(1)/to_R<R>(m.nom_size[e]));
      // 1/det from the float normals' determinant row (4 bytes per point, no conversion)
      if constexpr (DEF) mult *= R(1)/R(m.nrm[((size_t)(e - m.n_car)*(ND*ND + 1) + ND*ND)*nq + q]);
      if (compute_residual) {
        FaceT* rc = m.rcache + (size_t)e*nv*nq;
        #pragma unroll
        for (int v = 0; v < nv; ++v) rc[v*nq + q] = rc[v*nq + q] + tr[v]*mult;
      } else {
        #pragma unroll
        for (int v = 0; v < nv; ++v) st_w[v*nq + q] += f64_of(tr[v]*mult);
      }
    }
    #pragma unroll
    for (int v = 0; v < nv; ++v) my_u[v*nq + q] = offset_var<ND, R>(m, e, v, st_w[v*nq + q]);
  }
  __syncthreads();
  write_faces_from_smem<ND, RS, R, FaceT>(m, rt, s_u, e0, e_end);
}

// ------------------------------------------------------------------- Neighbor
// Element whose reference state the traces of a face slot are offsets from (mixed form).
template <int ND, typename FaceT>
__device__ __forceinline__ int slot_owner(const Dev<FaceT>& m, int slot)
{
  return slot < m.elem_slot_end ? slot/(2*ND) : m.slot_elem[slot - m.elem_slot_end];
}

// Spatial::Neighbor (include/Spatial.hpp:613-705): local Lax-Friedrichs flux written back
// to both faces with sign; LDG face average for the viscous path. One thread per face qpoint.
// same_ref: both slots are offsets from one reference (a boundary connection: the ghost face
// takes the inside element's).
template <int ND, int RS, typename R, typename FaceT>
__device__ __forceinline__ void neighbor_point(const Dev<FaceT>& m, int slot0, int slot1, int dir, int q,
                                               const FaceT* nrml, bool viscous, const double* ghost_override,
                                               bool same_ref)
{
  using S = Shape<ND, RS>;
  constexpr int nfq = S::nfq, nv = S::nv;
  // Mixed form: each side's traces are offsets from its own element's reference state. Side 1
  // is expressed in side 0's reference by adding the difference of the references, formed
  // from their float high and low parts (RefState::lo) so that it keeps float's relative
  // accuracy; the numerical flux is then the offset flux of side 0, and side 1 receives it
  // minus f(ref1).n - f(ref0).n, itself an offset flux. Nothing here needs double.
  constexpr bool split = !std::is_same<FaceT, double>::value;
  RefState<ND, R> rs;
  R delta[nv];   // ref1 - ref0
  bool cross = false;
  int e_ref = 0, e_ref1 = 0;
  if constexpr (split) {
    e_ref = slot_owner<ND>(m, slot0);
    e_ref1 = same_ref ? e_ref : slot_owner<ND>(m, slot1);
    const RefState<ND, R>* terms = reinterpret_cast<const RefState<ND, R>*>(m.ref_terms);
    rs = terms[e_ref];
    cross = e_ref1 != e_ref;
    if (cross) {
      const RefState<ND, R> r1 = terms[e_ref1];
      #pragma unroll
      for (int v = 0; v < nv; ++v) delta[v] = (r1.s[v] - rs.s[v]) + (r1.lo[v] - rs.lo[v]);
    } else {
      #pragma unroll
      for (int v = 0; v < nv; ++v) delta[v] = R(0);
    }
  }
  const bool deformed = nrml != nullptr;
  int sign0 = 1, sign1 = 1;
  if (deformed) {
    sign0 = 1 - 2*(((dir >> 4) & 1) == 0);
    sign1 = 1 - 2*(((dir >> 5) & 1) == 1);
  }
  const int q1 = deformed ? perm_index<ND, RS>(dir, q) : q;
  FaceT* f0 = m.face + (size_t)slot0*S::slot_dof;
  FaceT* f1 = m.face + (size_t)slot1*S::slot_dof;
  R o0[nv], o1[nv], jump[nv];   // offset-form traces (both from side 0's reference) and their jump
  #pragma unroll
  for (int v = 0; v < nv; ++v) {
    if constexpr (split) {
      o0[v] = R(f0[v*nfq + q]);
      o1[v] = ghost_override ? offset_var<ND, R>(m, e_ref, v, ghost_override[v]) : R(f1[v*nfq + q1]) + delta[v];
      jump[v] = o0[v] - o1[v];
    } else {
      const double a = double(f0[v*nfq + q]);
      const double b = ghost_override ? double(ghost_override[v]) : double(f1[v*nfq + q1]);
      o0[v] = R(a);
      o1[v] = R(b);
      jump[v] = R(a - b);
    }
  }
  if (viscous) {
    #pragma unroll
    for (int v = 0; v < nv; ++v) {
      R avg = R(.5)*(o0[v] + o1[v]);
      f0[nv*nfq + v*nfq + q] = FaceT(avg);
      f1[nv*nfq + v*nfq + q1] = FaceT(split ? avg - delta[v] : avg);
    }
    if (m.fta) return;   // Fix_therm_admis has no convection (Spatial.hpp:655-686 are skipped)
  }
  R u0[nv], u1[nv];
  #pragma unroll
  for (int v = 0; v < nv; ++v) {
    u0[v] = split ? rs.s[v] + o0[v] : o0[v];
    u1[v] = split ? rs.s[v] + o1[v] : o1[v];
  }
  R n[ND];
  const int i_dim0 = dir & 3;
  #pragma unroll
  for (int d = 0; d < ND; ++d) n[d] = deformed ? R(sign0)*R(nrml[d*nfq + q]) : (d == i_dim0 ? R(1) : R(0));
  R fl0[nv], fl1[nv], dref[nv];
  Conv<ND, R> c0(u0), c1(u1);
  if constexpr (split) {
    flux_delta<ND, R>(u0, o0, rs, c0.inv_mass, n, fl0);
    flux_delta<ND, R>(u1, o1, rs, c1.inv_mass, n, fl1);
    // f(ref1).n - f(ref0).n, the offset flux of side 1's reference from side 0's
    #pragma unroll
    for (int v = 0; v < nv; ++v) dref[v] = R(0);
    if (cross) {
      const RefState<ND, R> r1 = reinterpret_cast<const RefState<ND, R>*>(m.ref_terms)[e_ref1];
      flux_delta<ND, R>(r1.s, delta, rs, r1.inv_mass, n, dref);
    }
  } else {
    c0.flux(u0, n, fl0);
    c1.flux(u1, n, fl1);
  }
  const R cs0 = char_speed<ND, R>(u0, c0.inv_mass), cs1 = char_speed<ND, R>(u1, c1.inv_mass);
  R nn = 0;
  #pragma unroll
  for (int d = 0; d < ND; ++d) nn += n[d]*n[d];
  const R mult = fmax(cs0, cs1)*sqrt(nn);
  #pragma unroll
  for (int v = 0; v < nv; ++v) {
    R flux = R(.5)*(fl0[v] + fl1[v] + mult*jump[v]);
    f0[v*nfq + q] = FaceT(R(sign0)*flux);
    f1[v*nfq + q1] = FaceT(R(sign1)*(split ? flux - dref[v] : flux));
  }
}

// Calls f(connection, face point) for every face point of n_con connections, one per thread
// in a grid-stride loop. The float kernels use 32-bit unsigned indices (a constant divisor
// then costs a multiply-high; hexed_gpu_create refuses arenas with 2^31 face points or more,
// so the index and its stride stay below 2^32). The FP64 kernels (WIDE) keep 64-bit indices:
// with 32-bit ones their face kernel measured 4% slower (0.863 -> 0.900 ms on the 32^3 mesh).
template <int NFQ, bool WIDE, typename F>
__device__ __forceinline__ void for_face_points(int n_con, F&& f)
{
  if constexpr (WIDE) {
    const long total = (long)n_con*NFQ;
    for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x)
      f(int(t/NFQ), int(t%NFQ));
  } else {
    const unsigned total = unsigned(n_con)*NFQ, step = gridDim.x*blockDim.x;
    for (unsigned t = blockIdx.x*blockDim.x + threadIdx.x; t < total; t += step) f(int(t/NFQ), int(t%NFQ));
  }
}

// Calls f(connection, face point, record) like the 32-bit form of for_face_points, with the
// connection's record of 3 ints (slot, slot, orientation) from `con`. Each iteration loads
// the next iteration's record before it works its own face point, so that the gathers of
// the next iteration do not first wait for their record's load (float face kernels: 0.093
// -> 0.090 ms per Neighbor launch on the 32^3 Taylor-Green mesh, at 64 registers instead of
// 56, still 4 CTAs of 256 per SM).
template <int NFQ, typename F>
__device__ __forceinline__ void for_face_records(int n_con, const int* con, F&& f)
{
  const unsigned total = unsigned(n_con)*NFQ, step = gridDim.x*blockDim.x;
  unsigned t = blockIdx.x*blockDim.x + threadIdx.x;
  if (t >= total) return;
  unsigned i = t/NFQ;
  int rec[3] = {con[3*i], con[3*i + 1], con[3*i + 2]};
  while (true) {
    const unsigned tn = t + step;
    const bool more = tn < total;
    const unsigned in = more ? tn/NFQ : i;
    const int next[3] = {con[3*in], con[3*in + 1], con[3*in + 2]};
    f(int(i), int(t - i*NFQ), rec);
    if (!more) return;
    t = tn;
    i = in;
    #pragma unroll
    for (int k = 0; k < 3; ++k) rec[k] = next[k];
  }
}

template <int ND, int RS, typename R, bool DEF, bool VISC, typename FaceT>
__global__ void k_neighbor(Dev<FaceT> m)
{
  using S = Shape<ND, RS>;
  constexpr int nfq = S::nfq;
  auto work = [&](int i, int q, const int* c) {
    if constexpr (DEF)
      neighbor_point<ND, RS, R, FaceT>(m, c[0], c[1], c[2], q, m.def_con_nrml + (size_t)i*ND*nfq, VISC, nullptr,
                                       false);
    else
      neighbor_point<ND, RS, R, FaceT>(m, c[0], c[1], c[2] | (c[2] << 2) | (1 << 4), q, nullptr, VISC, nullptr,
                                       false);
  };
  const int n_con = DEF ? m.n_def_con : m.n_car_con;
  const int* con = DEF ? m.def_con : m.car_con;
  if constexpr (std::is_same<R, double>::value)
    for_face_points<nfq, true>(n_con, [&](int i, int q) { work(i, q, con + 3*i); });
  else
    for_face_records<nfq>(n_con, con, work);
}

// ------------------------------------------------------------------- boundary conditions
// Characteristics (include/pde.hpp:182-256) solved with partially pivoted LU; apply_char
// (src/Boundary_condition.cpp:82-95). Every loop is unrolled and the pivot row swaps are
// selects, so the 3x3 system stays in registers (no local-memory arrays), and divisions
// are reciprocal multiplies (one per pivot): on this part each warp-wide FP64 instruction
// holds an SM's FP64 pipe for many cycles, and boundary points run this per face point.
template <int ND, typename R = double>
struct Characteristics {
  R vals[3], vecs[3][3], dir[ND], mass, veloc[ND];
  R lu[3][3], inv_diag[3]; int piv[3];
  __device__ R nrml(const R* v) const
  {
    R r = 0;
    #pragma unroll
    for (int d = 0; d < ND; ++d) r += dir[d]*v[d];
    return r;
  }
  __device__ void tang(const R* v, R* out) const
  {
    R n = nrml(v);
    #pragma unroll
    for (int d = 0; d < ND; ++d) out[d] = v[d] - dir[d]*n;
  }
  __device__ Characteristics(const R* state, const R* direction)
  {
    R nsq = 0;
    #pragma unroll
    for (int d = 0; d < ND; ++d) nsq += direction[d]*direction[d];
    const R inv_norm = R(1)/sqrt(nsq);
    #pragma unroll
    for (int d = 0; d < ND; ++d) dir[d] = direction[d]*inv_norm;
    mass = state[ND];
    const R inv_mass = R(1)/mass;
    #pragma unroll
    for (int d = 0; d < ND; ++d) veloc[d] = state[d]*inv_mass;
    R vsq = 0;
    #pragma unroll
    for (int d = 0; d < ND; ++d) vsq += veloc[d]*veloc[d];
    R pres = R(.4)*(state[ND + 1] - R(.5)*mass*vsq);
    R sound_speed = sqrt(R(1.4)*fmax(pres, R(0))*inv_mass);
    vals[2] = nrml(veloc);
    vals[0] = vals[2] - sound_speed;
    vals[1] = vals[2] + sound_speed;
    #pragma unroll
    for (int sign = 0; sign < 2; ++sign) {
      R d_veloc = R(2*sign - 1)*sound_speed*inv_mass;
      R d_pres = R(1.4)*pres*inv_mass;
      vecs[0][sign] = vals[2] + mass*d_veloc;
      vecs[1][sign] = 1;
      vecs[2][sign] = d_pres/R(.4) + R(.5)*vsq + mass*vals[2]*d_veloc;
    }
    vecs[0][2] = vals[2];
    vecs[1][2] = 1;
    vecs[2][2] = R(.5)*vsq;
    #pragma unroll
    for (int i = 0; i < 3; ++i) {
      piv[i] = i;
      #pragma unroll
      for (int j = 0; j < 3; ++j) lu[i][j] = vecs[i][j];
    }
    #pragma unroll
    for (int k = 0; k < 3; ++k) {
      int p = k;
      R best = fabs(lu[k][k]);
      #pragma unroll
      for (int i = k + 1; i < 3; ++i) if (fabs(lu[i][k]) > best) { p = i; best = fabs(lu[i][k]); }
      #pragma unroll
      for (int i = k + 1; i < 3; ++i) {
        const bool sw = p == i;
        #pragma unroll
        for (int j = 0; j < 3; ++j) {
          const R a = lu[k][j], b = lu[i][j];
          lu[k][j] = sw ? b : a;
          lu[i][j] = sw ? a : b;
        }
        const int pa = piv[k], pb = piv[i];
        piv[k] = sw ? pb : pa;
        piv[i] = sw ? pa : pb;
      }
      inv_diag[k] = lu[k][k] != R(0) ? R(1)/lu[k][k] : R(0);
      #pragma unroll
      for (int i = k + 1; i < 3; ++i) {
        const R f = lu[i][k]*inv_diag[k];
        lu[i][k] = f;
        #pragma unroll
        for (int j = k + 1; j < 3; ++j) lu[i][j] -= f*lu[k][j];
      }
    }
  }
  __device__ void solve(const R* b, R* x) const
  {
    R y[3];
    #pragma unroll
    for (int i = 0; i < 3; ++i) {
      R acc = piv[i] == 0 ? b[0] : piv[i] == 1 ? b[1] : b[2];
      #pragma unroll
      for (int j = 0; j < i; ++j) acc -= lu[i][j]*y[j];
      y[i] = acc;
    }
    #pragma unroll
    for (int i = 2; i >= 0; --i) {
      R acc = y[i];
      #pragma unroll
      for (int j = i + 1; j < 3; ++j) acc -= lu[i][j]*x[j];
      x[i] = acc*inv_diag[i];
    }
  }
  __device__ void decomp(const R* state, R (*d)[3]) const
  {
    R mmtm[ND], tm[ND], tv[ND], corr[ND];
    #pragma unroll
    for (int i = 0; i < ND; ++i) mmtm[i] = state[i];
    tang(mmtm, tm);
    tang(veloc, tv);
    #pragma unroll
    for (int i = 0; i < ND; ++i) corr[i] = tm[i] - state[ND]*tv[i];
    R vc = 0;
    #pragma unroll
    for (int i = 0; i < ND; ++i) vc += veloc[i]*corr[i];
    R s1d[3] = {nrml(mmtm), state[ND], state[ND + 1] - vc};
    R eb[3];
    solve(s1d, eb);
    R ed[3][3];
    #pragma unroll
    for (int r = 0; r < 3; ++r)
      #pragma unroll
      for (int c = 0; c < 3; ++c) ed[r][c] = vecs[r][c]*eb[c];
    #pragma unroll
    for (int c = 0; c < 3; ++c) {
      d[ND][c] = ed[1][c];
      d[ND + 1][c] = ed[2][c];
      #pragma unroll
      for (int i = 0; i < ND; ++i) d[i][c] = dir[i]*ed[0][c] + tv[i]*eb[c];
    }
    #pragma unroll
    for (int i = 0; i < ND; ++i) d[i][2] += corr[i];
    d[ND + 1][2] += vc;
  }
};

template <int ND, typename R = double>
__device__ void apply_char(const R* state, const R* normal, int sign, const R* inside, const R* outside, R* out)
{
  constexpr int nv = ND + 2;
  Characteristics<ND, R> ch(state, normal);
  R di[nv][3], fo[nv][3];
  ch.decomp(inside, di);
  ch.decomp(outside, fo);
  #pragma unroll
  for (int i = 0; i < 3; ++i) {
    const bool take = sign*ch.vals[i] > 0;
    #pragma unroll
    for (int r = 0; r < nv; ++r) di[r][i] = take ? fo[r][i] : di[r][i];
  }
  #pragma unroll
  for (int r = 0; r < nv; ++r) { R acc = 0; for (int c = 0; c < 3; ++c) acc += di[r][c]; out[r] = acc; }
}

__device__ __forceinline__ double ipow_d(double x, int e) { double r = 1; for (int i = 0; i < e; ++i) r *= x; return r; }

template <int ND>
__device__ double ghost_heat_flux(const hexed_bc_spec& b, const double* s, double heat_flux)
{
  constexpr int nv = ND + 2;
  if (b.thermal_kind == HEXED_THERMAL_ENERGY) return heat_flux;
  if (b.thermal_kind == HEXED_THERMAL_HEAT_FLUX) return b.thermal_value;
  double temp = s[nv - 1]*.4/s[nv - 2]/specific_gas_air;
  const double sb = 2*ipow_d(3.14159265358979323846, 5)*ipow_d(1.380649e-23, 4)/(15*ipow_d(299792458., 2)*ipow_d(6.62607015e-34, 3));
  return b.emissivity*sb*ipow_d(temp, 4) + b.heat_transfer_coef*(temp - b.temperature);
}

// Flow_bc::apply_state for one face qpoint (src/Boundary_condition.cpp). Writes the ghost
// state into `gh` (registers) and the slot, and the state cache where the BC primes it.
template <int ND, int RS, typename FaceT>
__device__ void bc_state_point(const Dev<FaceT>& m, int i_bc, int q, double* gh)
{
  using S = Shape<ND, RS>;
  constexpr int nfq = S::nfq, nv = S::nv;
  const int* c = m.bc_con + 4*i_bc;
  const hexed_bc_spec& b = m.bc_spec[c[3]];
  const int ifs = (c[2] >> 2) & 1;
  FaceT* in = m.face + (size_t)c[0]*S::slot_dof;
  FaceT* gf = m.face + (size_t)c[1]*S::slot_dof;
  const double* nrml = m.bc_nrml + (size_t)i_bc*ND*nfq;
  double* sc = m.bc_cache + (size_t)i_bc*2*nv*nfq;
  constexpr bool split = !std::is_same<FaceT, double>::value;
  double ref[nv];   // offset of the stored traces (mixed form), see offset_var
  for (int v = 0; v < nv; ++v) ref[v] = !split ? 0. : m.ref[(size_t)(c[0]/(2*ND))*nv + v];
  double inside[nv], n[ND];
  for (int v = 0; v < nv; ++v) inside[v] = split ? double(in[v*nfq + q]) + ref[v] : double(in[v*nfq + q]);
  if (m.fta) {
    // Solver::fix_admissibility (src/Solver.cpp:1067-1072): ghost face = inside face
    for (int v = 0; v < nv; ++v) { gh[v] = inside[v]; gf[v*nfq + q] = in[v*nfq + q]; }
    return;
  }
  for (int d = 0; d < ND; ++d) n[d] = nrml[d*nfq + q];
  switch (b.kind) {
    case HEXED_BC_FREESTREAM:
      for (int v = 0; v < nv; ++v) gh[v] = b.freestream[v];
      break;
    case HEXED_BC_RIEMANN_INVARIANTS: {
      if constexpr (split) {
        // Mixed form: apply_char is linear in (inside, outside) for a fixed linearization
        // state and reproduces a state equal on both sides, so the ghost offset from the
        // reference is apply_char of the offsets; that runs in float with the accuracy of the
        // offsets. The clamps of the reference (src/Boundary_condition.cpp:126-130) replace
        // the offset only where they act.
        float d_in[nv], d_fs[nv], u_in[nv], nf[ND], st[nv], rf[nv];
        for (int v = 0; v < nv; ++v) {
          rf[v] = to_R<float>(ref[v]);
          d_in[v] = float(in[v*nfq + q]);
          d_fs[v] = to_R<float>(b.freestream[v] - ref[v]);
          u_in[v] = rf[v] + d_in[v];
        }
        for (int d = 0; d < ND; ++d) nf[d] = to_R<float>(n[d]);
        apply_char<ND, float>(u_in, nf, 1 - 2*ifs, d_in, d_fs, st);
        if (rf[ND] + st[ND] < u_in[ND]*.5f) st[ND] = u_in[ND]*.5f - rf[ND];
        float sq = 0.f, isq = 0.f;
        for (int d = 0; d < ND; ++d) { sq += (rf[d] + st[d])*(rf[d] + st[d]); isq += u_in[d]*u_in[d]; }
        const float kin = .5f*sq/(rf[ND] + st[ND]);
        const float ikin = .5f*isq/u_in[ND];
        const float half_int = (u_in[ND + 1] - ikin)*.5f;
        if (rf[ND + 1] + st[ND + 1] - kin < half_int) st[ND + 1] = fmaxf(kin + half_int, 0.f) - rf[ND + 1];
        for (int v = 0; v < nv; ++v) { gh[v] = ref[v] + f64_of(st[v]); sc[v*nfq + q] = inside[v]; }
        break;
      }
      double st[nv];
      apply_char<ND>(inside, n, 1 - 2*ifs, inside, b.freestream, st);
      st[ND] = fmax(st[ND], inside[ND]/2);
      double sq = 0., isq = 0.;
      for (int d = 0; d < ND; ++d) { sq += st[d]*st[d]; isq += inside[d]*inside[d]; }
      double kin = .5*sq/st[ND];
      double ikin = .5*isq/inside[ND];
      st[ND + 1] = fmax(kin + fmax(st[ND + 1] - kin, (inside[ND + 1] - ikin)/2), 0.);
      for (int v = 0; v < nv; ++v) { gh[v] = st[v]; sc[v*nfq + q] = inside[v]; }
      break;
    }
    case HEXED_BC_NONPENETRATION: {
      double dot = 0., norm_sq = 0.;
      for (int d = 0; d < ND; ++d) { dot += inside[d]*n[d]; norm_sq += n[d]*n[d]; }
      for (int v = 0; v < nv; ++v) gh[v] = inside[v];
      for (int d = 0; d < ND; ++d) gh[d] -= 2*dot*n[d]/norm_sq;
      break;
    }
    case HEXED_BC_COPY:
    case HEXED_BC_OUTFLOW:
      for (int v = 0; v < nv; ++v) { gh[v] = inside[v]; gf[nv*nfq + v*nfq + q] = in[nv*nfq + v*nfq + q]; }
      break;
    case HEXED_BC_PRESSURE_OUTFLOW: {
      const int sign = 2*ifs - 1;
      double dot = 0., nsq = 0., msq = 0.;
      for (int d = 0; d < ND; ++d) { dot += inside[d]*n[d]; nsq += n[d]*n[d]; msq += inside[d]*inside[d]; }
      double nrml_veloc = dot/inside[ND]/sqrt(nsq);
      double kin = .5*msq/inside[ND];
      double pres = fmax(.4*(inside[ND + 1] - kin), 0.);
      double sound = sqrt(1.4*pres/inside[ND]);
      for (int v = 0; v < nv; ++v) gh[v] = inside[v];
      if (nrml_veloc*sign < sound) gh[ND + 1] = b.pressure/.4 + kin;
      break;
    }
    case HEXED_BC_NO_SLIP: {
      for (int d = 0; d < ND; ++d) gh[d] = -inside[d];
      gh[ND] = inside[ND];
      double ge = (b.thermal_kind == HEXED_THERMAL_ENERGY) ? b.thermal_value*inside[ND] : inside[ND + 1];
      gh[ND + 1] = ge*ge/inside[nv - 1];
      for (int v = 0; v < nv; ++v) sc[v*nfq + q] = (gh[v] + inside[v])/2;
      break;
    }
    default:
      for (int v = 0; v < nv; ++v) gh[v] = inside[v];
      break;
  }
  for (int v = 0; v < nv; ++v) gf[v*nfq + q] = FaceT(split ? gh[v] - ref[v] : gh[v]);
}

template <int ND, int RS, typename FaceT>
__global__ void k_bc_state(Dev<FaceT> m)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  const long total = (long)m.n_bc_con*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    double gh[ND + 2];
    bc_state_point<ND, RS, FaceT>(m, int(t/nfq), int(t%nfq), gh);
  }
}

// Neighbor over boundary connections; with FUSE the state BC is applied first in the same
// thread (Solver::apply_state_bcs followed by the boundary part of Neighbor).
template <int ND, int RS, typename R, bool VISC, bool FUSE, typename FaceT>
__global__ void k_bc_neighbor(Dev<FaceT> m)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  for_face_points<nfq, std::is_same<R, double>::value>(m.n_bc_con, [&](int i, int q) {
    const int* c = m.bc_con + 4*i;
    double gh[ND + 2];
    const double* ov = nullptr;
    if (FUSE) {
      bc_state_point<ND, RS, FaceT>(m, i, q, gh);
      ov = gh;
    }
    neighbor_point<ND, RS, R, FaceT>(m, c[0], c[1], bc_dir(c[2]), q, m.bc_nrml_t + (size_t)i*ND*nfq, VISC, ov, true);
  });
}

// Neighbor of a Cartesian-only mesh in one launch: blocks [0, car_blocks) take the Cartesian
// connections (as k_neighbor), the remaining blocks the boundary connections (as
// k_bc_neighbor) with one warp each. Same per-point arithmetic, one launch fewer per stage.
// The boundary condition is long double-precision code, and on a small mesh its points would
// otherwise sit in one CTA, bound by a single SM's FP64 throughput; one warp per CTA spreads
// them over as many SMs as there are warps of points.
constexpr int bc_warp = 32;
template <int ND, int RS, typename R, bool VISC, bool FUSE, typename FaceT>
__global__ void k_neighbor_car_bc(Dev<FaceT> m, int car_blocks)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  // 32-bit unsigned face-point indices (see for_face_points)
  if ((int)blockIdx.x < car_blocks) {
    const unsigned total = unsigned(m.n_car_con)*nfq, step = unsigned(car_blocks)*blockDim.x;
    for (unsigned t = blockIdx.x*blockDim.x + threadIdx.x; t < total; t += step) {
      const int i = int(t/nfq), q = int(t%nfq);
      const int* c = m.car_con + 3*i;
      neighbor_point<ND, RS, R, FaceT>(m, c[0], c[1], c[2] | (c[2] << 2) | (1 << 4), q, nullptr, VISC, nullptr,
                                       false);
    }
  } else {
    if ((int)threadIdx.x >= bc_warp) return;
    const unsigned total = unsigned(m.n_bc_con)*nfq, stride = unsigned(gridDim.x - car_blocks)*bc_warp;
    for (unsigned t = (blockIdx.x - car_blocks)*unsigned(bc_warp) + threadIdx.x; t < total; t += stride) {
      const int i = int(t/nfq), q = int(t%nfq);
      const int* c = m.bc_con + 4*i;
      double gh[ND + 2];
      const double* ov = nullptr;
      if (FUSE) {
        bc_state_point<ND, RS, FaceT>(m, i, q, gh);
        ov = gh;
      }
      neighbor_point<ND, RS, R, FaceT>(m, c[0], c[1], bc_dir(c[2]), q, m.bc_nrml_t + (size_t)i*ND*nfq, VISC, ov, true);
    }
  }
}

// Solver::apply_flux_bcs (src/Solver.cpp:69-81) + Flow_bc::apply_flux.
template <int ND, int RS, typename FaceT>
__device__ void bc_flux_point(const Dev<FaceT>& m, int i_bc, int q)
{
  using S = Shape<ND, RS>;
  constexpr int nfq = S::nfq, nv = S::nv;
  const int* c = m.bc_con + 4*i_bc;
  const hexed_bc_spec& b = m.bc_spec[c[3]];
  const int ifs = (c[2] >> 2) & 1;
  FaceT* in_l = m.face + (size_t)c[0]*S::slot_dof + nv*nfq;
  FaceT* gh_l = m.face + (size_t)c[1]*S::slot_dof + nv*nfq;
  if (m.fta) {
    // Solver::apply_fta_flux_bcs (src/Solver.cpp:103-114): ghost LDG flux = -inside
    for (int v = 0; v < nv; ++v) gh_l[v*nfq + q] = -in_l[v*nfq + q];
    return;
  }
  const double* nrml = m.bc_nrml + (size_t)i_bc*ND*nfq;
  double* sc = m.bc_cache + (size_t)i_bc*2*nv*nfq;
  double* fc = sc + nv*nfq;
  double in[nv], n[ND];
  for (int v = 0; v < nv; ++v) { in[v] = double(in_l[v*nfq + q]); fc[v*nfq + q] = in[v]; }
  for (int d = 0; d < ND; ++d) n[d] = nrml[d*nfq + q];
  double out[nv];
  switch (b.kind) {
    case HEXED_BC_FREESTREAM:
    case HEXED_BC_COPY: {
      FaceT* in_s = m.face + (size_t)c[0]*S::slot_dof;
      FaceT* gh_s = m.face + (size_t)c[1]*S::slot_dof;
      for (int v = 0; v < nv; ++v) gh_s[v*nfq + q] = in_s[v*nfq + q];
      for (int v = 0; v < nv; ++v) out[v] = in[v];
      break;
    }
    case HEXED_BC_RIEMANN_INVARIANTS: {
      double cache[nv], zero[nv];
      for (int v = 0; v < nv; ++v) { cache[v] = sc[v*nfq + q]; zero[v] = 0.; }
      apply_char<ND>(cache, n, 1 - 2*ifs, zero, in, out);
      break;
    }
    case HEXED_BC_NONPENETRATION: {
      for (int v = 0; v < nv; ++v) out[v] = -in[v];
      double dot = 0., norm_sq = 0.;
      for (int d = 0; d < ND; ++d) { dot += out[d]*n[d]; norm_sq += n[d]*n[d]; }
      for (int d = 0; d < ND; ++d) out[d] -= 2*dot*n[d]/norm_sq;
      break;
    }
    case HEXED_BC_OUTFLOW:
    case HEXED_BC_PRESSURE_OUTFLOW:
      for (int v = 0; v < nv; ++v) out[v] = -in[v];
      break;
    case HEXED_BC_NO_SLIP: {
      for (int d = 0; d < ND; ++d) out[d] = in[d];
      out[ND] = -in[ND];
      double normal = 0;
      for (int d = 0; d < ND; ++d) normal += n[d]*n[d];
      normal = sqrt(normal);
      const int flux_sign = 2*ifs - 1;
      double s[nv];
      for (int v = 0; v < nv; ++v) s[v] = sc[v*nfq + q];
      const double x = in[ND + 1];
      out[ND + 1] = b.coercion*(normal*flux_sign*ghost_heat_flux<ND>(b, s, x*flux_sign/normal) - x) + x;
      break;
    }
    default:
      for (int v = 0; v < nv; ++v) out[v] = in[v];
  }
  for (int v = 0; v < nv; ++v) gh_l[v*nfq + q] = FaceT(out[v]);
}

// Neighbor_reconcile (include/Spatial.hpp:716-759) for one face qpoint.
template <int ND, int RS, typename R, typename FaceT>
__device__ __forceinline__ void reconcile_point(const Dev<FaceT>& m, int slot0, int slot1, int dir, int q, bool deformed)
{
  using S = Shape<ND, RS>;
  constexpr int nfq = S::nfq, nv = S::nv;
  int sign0 = 1, sign1 = 1;
  if (deformed) {
    sign0 = 1 - 2*(((dir >> 4) & 1) == 0);
    sign1 = 1 - 2*(((dir >> 5) & 1) == 1);
  }
  const int q1 = deformed ? perm_index<ND, RS>(dir, q) : q;
  FaceT* l0 = m.face + (size_t)slot0*S::slot_dof + nv*nfq;
  FaceT* l1 = m.face + (size_t)slot1*S::slot_dof + nv*nfq;
  #pragma unroll
  for (int v = 0; v < nv; ++v) {
    R a = R(l0[v*nfq + q]), b = R(l1[v*nfq + q1]);
    R avg = 0;
    avg += R(.5*sign0)*a;
    avg += R(.5*sign1)*b;
    l0[v*nfq + q] = FaceT(R(sign0)*avg - a);
    l1[v*nfq + q1] = FaceT(R(sign1)*avg - b);
  }
}

template <int ND, int RS, typename R, int KIND, bool FUSE_BC, typename FaceT>  // KIND 0 car, 1 def, 2 bc
__global__ void k_neighbor_reconcile(Dev<FaceT> m)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  const int n_con = KIND == 0 ? m.n_car_con : KIND == 1 ? m.n_def_con : m.n_bc_con;
  if constexpr (KIND < 2 && !std::is_same<R, double>::value) {
    for_face_records<nfq>(n_con, KIND == 0 ? m.car_con : m.def_con, [&](int, int q, const int* c) {
      reconcile_point<ND, RS, R, FaceT>(m, c[0], c[1], KIND == 0 ? 0 : c[2], q, KIND == 1);
    });
    return;
  }
  for_face_points<nfq, std::is_same<R, double>::value>(n_con, [&](int i, int q) {
    if (KIND == 0) {
      const int* c = m.car_con + 3*i;
      reconcile_point<ND, RS, R, FaceT>(m, c[0], c[1], 0, q, false);
    } else if (KIND == 1) {
      const int* c = m.def_con + 3*i;
      reconcile_point<ND, RS, R, FaceT>(m, c[0], c[1], c[2], q, true);
    } else {
      const int* c = m.bc_con + 4*i;
      if (FUSE_BC) bc_flux_point<ND, RS, FaceT>(m, i, q);
      reconcile_point<ND, RS, R, FaceT>(m, c[0], c[1], bc_dir(c[2]), q, true);
    }
  });
}

template <int ND, int RS, typename FaceT>
__global__ void k_bc_flux(Dev<FaceT> m)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  const long total = (long)m.n_bc_con*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x)
    bc_flux_point<ND, RS, FaceT>(m, int(t/nfq), int(t%nfq));
}

// ------------------------------------------------------------------- hanging faces
// Prolong_refined / Restrict_refined (include/Spatial.hpp:153-285) of one refined face (the
// calling CTA): NVAR face variables of the slots of `base` (slot_stride values per slot), the
// LDG half starting ldg_offset values into a slot. Thread (fine face, var, qpoint); row
// transforms go through shared memory one dimension at a time. The flow uses the arena's face
// slots with its nv variables; the smoothness-based AV uses its own slots and variable counts.
template <int ND, int RS, bool PROLONG, int NVAR, typename FaceT>
__device__ __forceinline__ void refine_face(FaceT* base, size_t slot_stride, int ldg_offset, const int* rf,
                                            const Tab<RS>& tab, int scale, int offset)
{
  using S = Shape<ND, RS>;
  constexpr int nfq = S::nfq;
  constexpr int n_face = 1 << (ND - 1);
  __shared__ double s_face[n_face*NVAR*nfq];
  __shared__ double s_mat[2*RS*RS];
  for (int i = threadIdx.x; i < 2*RS*RS; i += blockDim.x) s_mat[i] = PROLONG ? tab.prolong[i] : tab.restrict_[i];
  const bool str[2] = {rf[5] != 0, rf[6] != 0};
  int nf = n_face;
  for (int d = 0; d < ND - 1; ++d) nf /= 1 + str[d];
  FaceT* coarse = base + (size_t)rf[0]*slot_stride + offset*ldg_offset;
  const int n_item = nf*NVAR*nfq;
  __syncthreads();
  for (int t = threadIdx.x; t < n_item; t += blockDim.x) {
    const int i_face = t/(NVAR*nfq), k = t%(NVAR*nfq);
    FaceT* fine = base + (size_t)rf[1 + i_face]*slot_stride + offset*ldg_offset;
    s_face[t] = PROLONG ? double(coarse[k]) : double(fine[k]);
  }
  #pragma unroll 1
  for (int d = 0; d < ND - 1; ++d) {
    __syncthreads();
    double val[(n_face*NVAR*nfq + 63)/64 + 1];
    int cnt = 0;
    for (int t = threadIdx.x; t < n_item; t += blockDim.x, ++cnt) {
      const int i_face = t/(NVAR*nfq), k = t%(NVAR*nfq);
      const int qq = k%nfq;
      double x = s_face[t];
      if (str[d]) {
        x = PROLONG ? x*double(1 + scale) : x/double(1 + scale);
      } else {
        const int pw = ND - 2 - d;
        const int face_stride = str[ND - 2] ? 1 : ipow(2, pw);
        const int qstride = ipow(RS, pw);
        const int i_half = (i_face/face_stride)%2;
        const int i = (qq/qstride)%RS;
        const int row0 = t - i*qstride;
        const double* mat = s_mat + i_half*RS*RS;
        double acc = 0.;
        #pragma unroll
        for (int j = 0; j < RS; ++j) acc += mat[i*RS + j]*s_face[row0 + j*qstride];
        x = acc;
      }
      val[cnt] = x;
    }
    __syncthreads();
    cnt = 0;
    for (int t = threadIdx.x; t < n_item; t += blockDim.x, ++cnt) s_face[t] = val[cnt];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < n_item; t += blockDim.x) {
    const int i_face = t/(NVAR*nfq), k = t%(NVAR*nfq);
    FaceT* fine = base + (size_t)rf[1 + i_face]*slot_stride + offset*ldg_offset;
    fine[k] = FaceT(s_face[t]);
  }
  if (!PROLONG) {
    for (int k = threadIdx.x; k < NVAR*nfq; k += blockDim.x) {
      double acc = 0.;
      for (int i_face = 0; i_face < nf; ++i_face) acc += s_face[i_face*NVAR*nfq + k];
      coarse[k] = FaceT(acc);
    }
  }
}

// One CTA per refined face of the arena's face slots.
template <int ND, int RS, bool PROLONG, typename FaceT>
__global__ void k_refine(Dev<FaceT> m, Tab<RS> tab, int scale, int offset)
{
  using S = Shape<ND, RS>;
  refine_face<ND, RS, PROLONG, S::nv, FaceT>(m.face, S::slot_dof, S::nv*S::nfq, m.ref_face + 7*blockIdx.x, tab,
                                             scale, offset);
}

// ------------------------------------------------------------------- Write_face (standalone)
template <int ND, int RS, typename FaceT>
__global__ void k_write_face(Dev<FaceT> m, Tab<RS> tab, int e_begin, int n_elem)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  const long total = (long)n_elem*ND*nv*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    int r = int(t%nfq); long rest = t/nfq;
    int v = int(rest%nv); rest /= nv;
    int d = int(rest%ND); int e = e_begin + int(rest/ND);
    const int stride = S::stride(d);
    const double* row = m.elem + (size_t)e*(nv + 3)*nq + v*nq + (r/stride)*stride*RS + r%stride;
    // traces in the offset form of the storage (see offset_var)
    const double ref = std::is_same<FaceT, double>::value ? 0. : m.ref[(size_t)e*nv + v];
    double a0 = 0., a1 = 0.;
    for (int i = 0; i < RS; ++i) { double x = row[i*stride] - ref; a0 += tab.bound[i]*x; a1 += tab.bound[RS + i]*x; }
    FaceT* f0 = m.face + (size_t)(e*2*ND + 2*d)*S::slot_dof + v*nfq + r;
    f0[0] = FaceT(a0);
    f0[S::slot_dof] = FaceT(a1);
  }
}

// ------------------------------------------------------------------- Max_dt
// Spatial::Max_dt (include/Spatial.hpp:784-828); global minimum through per-CTA partials.
// R is the compute type: double for the FP64 form; float for the mixed form, whose time
// step is a CFL limit with a safety factor and needs no more than float accuracy.
// Each CTA writes its minimum to partials and takes a ticket; the CTA that takes the last one
// (all partials written and fenced before it) forms the minimum over the partials, the
// stage's step dt = min(max_dt, max_time_step)*cheby (src/Solver.cpp:843-846; max_dt is 1
// under local time stepping) into scalars, and resets the ticket. No CTA waits on another.
template <int ND, int RS, typename R, bool VISC, typename FaceT>
__global__ void __launch_bounds__(256)
k_max_dt(Dev<FaceT> m, Tab<RS> tab, R inv_cfl_c, R inv_cfl_d, int local_time, TmT<R> visc, TmT<R> cond,
         double* partials, unsigned* ticket, double max_time_step, double cheby)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nv = S::nv;
  __shared__ R s_node[RS];
  if (threadIdx.x < RS) s_node[threadIdx.x] = to_R<R>(tab.node[threadIdx.x]);
  __syncthreads();
  double dt = 1.7976931348623157e308;
  R dt_r = R(3.4e38);   // running minimum in the compute type (float form)
  // 32-bit unsigned point index: hexed_gpu_create refuses arenas of 2^31 points or more
  const unsigned total = unsigned(m.n_elem)*nq, step = gridDim.x*blockDim.x;
  for (unsigned t = blockIdx.x*blockDim.x + threadIdx.x; t < total; t += step) {
    const int e = int(t/nq), q = int(t%nq);
    double* state = m.elem + (size_t)e*(nv + 3)*nq;
    R coord[ND];
    point_coords<ND, RS>(s_node, q, coord);
    if constexpr (std::is_same<R, double>::value) {
      const double step = point_step<ND, RS, R, VISC>(m, e, q, coord, inv_cfl_c, inv_cfl_d, visc, cond);
      if (local_time) state[nv*nq + q] = step;
      else {
        state[nv*nq + q] = 1.;
        dt = fmin(dt, step);
      }
    } else {
      const R step = point_step<ND, RS, R, VISC>(m, e, q, coord, inv_cfl_c, inv_cfl_d, visc, cond);
      if (local_time) state[nv*nq + q] = f64_of(step);
      else {
        state[nv*nq + q] = 1.;
        dt_r = fmin(dt_r, step);
      }
    }
  }
  if constexpr (!std::is_same<R, double>::value) dt = dt_r < R(3.4e38) ? f64_of(dt_r) : dt;
  // CTA minimum
  __shared__ double s_min[32];
  for (int o = 16; o > 0; o >>= 1) dt = fmin(dt, __shfl_xor_sync(0xffffffffu, dt, o));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = dt;
  __syncthreads();
  __shared__ bool s_last;
  if (threadIdx.x < 32) {
    double x = threadIdx.x < (blockDim.x + 31)/32 ? s_min[threadIdx.x] : 1.7976931348623157e308;
    for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = x;
      __threadfence();
      s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!s_last) return;
  // the last CTA: minimum over every CTA's partial (read past L1), in any order (fmin is exact)
  __threadfence();
  // one running minimum, the loop unrolled so that its loads overlap (a wider tail would raise
  // the register count of the whole kernel)
  double y = 1.7976931348623157e308;
  #pragma unroll 4
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) y = fmin(y, __ldcg(partials + i));
  for (int o = 16; o > 0; o >>= 1) y = fmin(y, __shfl_xor_sync(0xffffffffu, y, o));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = y;   // warp 0 read s_min before the barrier
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 1.7976931348623157e308;
    for (int i = 0; i < (int)(blockDim.x + 31)/32; ++i) r = fmin(r, s_min[i]);
    if (local_time) r = 1.;
    m.scalars[SC_MAXDT] = r;
    m.scalars[SC_DT] = fmin(r, max_time_step)*cheby;
    *ticket = 0u;
  }
}

static __global__ void k_set_scalar(double* scalars, int which, double value) { scalars[which] = value; }
static __global__ void k_copy_scalars(double* scalars, int from, int to, int n)
{
  for (int i = threadIdx.x; i < n; i += blockDim.x) scalars[to + i] = scalars[from + i];
}

// thermo::admissible (src/thermo.cpp:6-18) over every element state, every element face trace
// and every fine mortar face, as Solver::is_admissible does (src/Solver.cpp:921-959): density
// and total energy positive at every point. record[e] = 1 marks an inadmissible element (its
// state or one of its faces); status bit 0 is set if any point is inadmissible, bit 1 if any
// value is not finite (the reference asserts there). Traces of the mixed form are offsets:
// the element's reference state is added back.
template <int ND, int RS, typename FaceT>
__global__ void k_admissible(Dev<FaceT> m, int* record, int* status)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  constexpr bool split = !std::is_same<FaceT, double>::value;
  const long n_state = (long)m.n_elem*nq;
  const long n_face = (long)m.n_elem*2*ND*nfq;
  const long n_mortar = (long)m.n_ref*4*nfq;
  const long total = n_state + n_face + n_mortar;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    double val[nv];
    int e;
    if (t < n_state) {
      e = int(t/nq);
      const int q = int(t%nq);
      const double* st = m.elem + (size_t)e*(nv + 3)*nq;
      for (int v = 0; v < nv; ++v) val[v] = st[v*nq + q];
    } else {
      int slot, r;
      if (t < n_state + n_face) {
        const long u = t - n_state;
        slot = int(u/nfq);
        r = int(u%nfq);
        e = slot/(2*ND);
      } else {
        const long u = t - n_state - n_face;
        const int i = int(u/(4*nfq)), k = int((u/nfq)%4);
        r = int(u%nfq);
        const int* rf = m.ref_face + 7*i;
        int n_fine = 1 << (ND - 1);
        for (int d = 0; d < ND - 1; ++d) n_fine /= 1 + (rf[5 + d] != 0);
        if (k >= n_fine || rf[1 + k] < 0) continue;
        slot = rf[1 + k];
        e = -1;   // a mortar belongs to no element; its reference is the coarse element's
        if constexpr (split) e = rf[0]/(2*ND);
      }
      const FaceT* f = m.face + (size_t)slot*S::slot_dof;
      for (int v = 0; v < nv; ++v) {
        val[v] = double(f[v*nfq + r]);
        if constexpr (split) val[v] += m.ref[(size_t)e*nv + v];
      }
      if (t >= n_state + n_face) e = -1;
    }
    bool finite = true;
    for (int v = 0; v < nv; ++v) finite = finite && isfinite(val[v]);
    const bool admissible = val[ND] > 0. && val[ND + 1] > 0.;
    if (!finite) atomicOr(status, 2);
    if (!admissible) {
      atomicOr(status, 1);
      if (e >= 0) record[e] = 1;
    }
  }
}

// Storage conversions of the mixed form and the determinant reciprocal.
static __global__ void k_narrow(const double* src, float* dst, long n)
{
  for (long i = blockIdx.x*(long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x*blockDim.x) dst[i] = float(src[i]);
}
static __global__ void k_widen(const float* src, double* dst, long n)
{
  for (long i = blockIdx.x*(long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x*blockDim.x) dst[i] = double(src[i]);
}
// Conserved rows [n][row] of a contiguous staging buffer into the element array, whose
// elements are `pitch` doubles apart (hexed_gpu_write_state: the host copy goes to the
// staging buffer as one contiguous transfer).
static __global__ void k_scatter_rows(const double* stage, double* elem, long n, int row, int pitch)
{
  const long total = n*row;
  for (long i = blockIdx.x*(long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x*blockDim.x) {
    const long e = i/row, r = i%row;
    elem[e*pitch + r] = stage[i];
  }
}
static __global__ void k_inv_det(const double* jac, double* inv_det, long n_def, int nq, int n_metric)
{
  const long n = n_def*nq;
  for (long i = blockIdx.x*(long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x*blockDim.x) {
    const long e = i/nq, q = i%nq;
    inv_det[i] = 1./jac[(e*(n_metric + 1) + n_metric)*nq + q];
  }
}

// FP64 pipe probe: fp64_fma_chains independent dependent-FMA chains per thread.
constexpr int fp64_fma_chains = 8;
static __global__ void k_fp64_fma(double* out, int iters, double a)
{
  double x[fp64_fma_chains];
  #pragma unroll
  for (int k = 0; k < fp64_fma_chains; ++k) x[k] = threadIdx.x*1e-3 + k;
  for (int i = 0; i < iters; ++i) {
    #pragma unroll
    for (int k = 0; k < fp64_fma_chains; ++k) x[k] = fma(x[k], a, 1e-7);
  }
  double s = 0.;
  #pragma unroll
  for (int k = 0; k < fp64_fma_chains; ++k) s += x[k];
  out[blockIdx.x*blockDim.x + threadIdx.x] = s;
}

// ------------------------------------------------------------------- artificial viscosity
// Stab_art_visc (src/stabilizing_art_visc.cpp:26-60): per-element smoothness indicator of the
// specific volume. One warp per element, with no block-wide barrier past the tables: each lane
// takes the points lane, lane + 32, ..., stores their specific volumes in the warp's shared row
// and sums their terms of the norm; after a warp barrier the lanes take the nd*nfq rows the same
// way, each row's squared projection onto the highest Legendre mode; the warp then reduces both
// sums by shuffles
// (the reference sums in sequence: the two orders differ in the last bits). R is the type of the
// terms and sums: double in the FP64 form, float in the mixed form, whose coefficient only has to
// hold the mixed form's tolerance.
constexpr int av_warps = 8;   // elements per CTA of k_av_uncert

// The basis values the artificial-viscosity kernels use, already in their type R (rounded to
// nearest on the host for the mixed form), so that no conversion runs per point or per row:
// w = quadrature weights, ow = highest orthonormal Legendre mode times the weight, node = nodes.
template <int RS, typename R>
struct AvTab { R w[RS]; R ow[RS]; R node[RS]; };

// The indicator's ramp in log10 of the non-smoothness (src/stabilizing_art_visc.cpp:47-55):
// centre -4.25 log10(row_size - 1), half width 0.5; lo and hi are 10^(centre -+ half width),
// the ratio's bounds below and above which the indicator is 0 and 1.
struct AvRamp { double center, half_width, lo, hi; };

template <int ND, int RS, typename R>
__global__ void __launch_bounds__(av_warps*32)
k_av_uncert(const double* elem, const double* nom_size, int n_elem, AvTab<RS, R> tab, double char_speed, AvRamp ramp,
            double* uncert)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nv = S::nv;
  constexpr int ppl = (nq + 31)/32;   // points per lane
  __shared__ R s_iv[av_warps][nq];
  __shared__ R s_w[RS], s_ow[RS];
  // the tables go to shared memory by constant indices: indexing the parameter by a lane's
  // point would copy it to local memory in every thread
  if (threadIdx.x == 0) {
    #pragma unroll
    for (int i = 0; i < RS; ++i) { s_w[i] = tab.w[i]; s_ow[i] = tab.ow[i]; }
  }
  __syncthreads();   // the only block-wide barrier
  const int warp = threadIdx.x/32, lane = threadIdx.x%32;
  const int e = blockIdx.x*av_warps + warp;
  if (e >= n_elem) return;   // whole warps leave
  const double* rho = elem + (size_t)e*(nv + 3)*nq + ND*nq;
  R* iv = s_iv[warp];
  double r[ppl];
  #pragma unroll
  for (int k = 0; k < ppl; ++k) r[k] = lane + 32*k < nq ? rho[lane + 32*k] : 1.;
  R sn = 0;
  #pragma unroll
  for (int k = 0; k < ppl; ++k) {
    const int q = lane + 32*k;
    if (q >= nq) break;
    const R v = std::is_same<R, double>::value ? R(1./r[k]) : R(1)/to_R<R>(r[k]);
    iv[q] = v;
    R w = 1;
    #pragma unroll
    for (int d = 0; d < ND; ++d) w *= s_w[(q/ipow(RS, ND - 1 - d))%RS];
    sn += v*v*w;
  }
  __syncwarp();
  R sr = 0;
  for (int t = lane; t < ND*nfq; t += 32) {
    const int d = t/nfq, rr = t%nfq;
    const int stride = S::stride(d);
    const R* row = iv + (rr/stride)*stride*RS + rr%stride;
    R dot = 0;
    #pragma unroll
    for (int i = 0; i < RS; ++i) dot += row[i*stride]*s_ow[i];
    R fw = 1;
    #pragma unroll
    for (int k = 0; k < ND - 1; ++k) fw *= s_w[(rr/ipow(RS, ND - 2 - k))%RS];
    sr += dot*dot*fw;
  }
  #pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sn += __shfl_xor_sync(0xffffffffu, sn, o);
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
  }
  if (lane) return;
  // below and above the ramp by the thresholds on the ratio itself, without the division and the
  // logarithm; the ramp (and a NaN) as the reference forms it
  const double num = double(sr), den = double(sn)*ND;
  double indicator;
  if (den > 0 && num <= ramp.lo*den) indicator = 0;
  else if (den > 0 && num >= ramp.hi*den) indicator = 1;
  else {
    indicator = log(num/den)/log(10.);
    if (indicator <= ramp.center - ramp.half_width) indicator = 0;
    else if (indicator < ramp.center + ramp.half_width)
      indicator = .5*(1 + sin(3.14159265358979323846*(indicator - ramp.center)/2/ramp.half_width));
    else indicator = 1;
  }
  uncert[e] = (RS - 1)*char_speed*nom_size[e]*indicator;
}

// share_vertex_data with Vertex::vector_max (src/Solver.cpp:35-54): the values are >= 0, so
// their IEEE bit patterns order like the values and an integer atomicMax takes the maximum.
template <int ND>
__global__ void k_av_vertex_max(const int* vert_id, int n_elem, const double* uncert, double* vmax)
{
  constexpr int nvert = 1 << ND;
  const long total = (long)n_elem*nvert;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const double x = uncert[t/nvert];
    atomicMax(reinterpret_cast<unsigned long long*>(vmax) + vert_id[t], (unsigned long long)__double_as_longlong(x));
  }
}

// Solver::fix_admissibility's vertex coefficient (src/Solver.cpp:990-1008): an element's
// admissibility record as the value its vertices start from ...
static __global__ void k_record_to_value(const int* record, int n_elem, double* out)
{
  for (int e = blockIdx.x*blockDim.x + threadIdx.x; e < n_elem; e += gridDim.x*blockDim.x) out[e] = record[e];
}

// ... and, after the first vertex maximum, the maximum over each element's vertices
template <int ND>
__global__ void k_elem_vertex_max(const int* vert_id, int n_elem, const double* vmax, double* out)
{
  constexpr int nvert = 1 << ND;
  for (int e = blockIdx.x*blockDim.x + threadIdx.x; e < n_elem; e += gridDim.x*blockDim.x) {
    double x = 0;
    for (int v = 0; v < nvert; ++v) x = fmax(x, vmax[vert_id[e*nvert + v]]);
    out[e] = x;
  }
}

// std::swap of the bulk and Laplacian artificial-viscosity rows of every qpoint
// (src/Solver.cpp:1033-1039, 1083-1089)
template <int ND, int RS>
__global__ void k_swap_av(double* elem, int n_elem)
{
  constexpr int nq = Shape<ND, RS>::nq, nv = Shape<ND, RS>::nv;
  const long total = (long)n_elem*nq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    double* st = elem + (size_t)(t/nq)*(nv + 3)*nq + t%nq;
    const double b = st[(nv + 1)*nq];
    st[(nv + 1)*nq] = st[(nv + 2)*nq];
    st[(nv + 2)*nq] = b;
  }
}

// Multilinear interpolation of the vertex values to the qpoints (Gauss_lobatto(2).interpolate
// + math::hypercube_matvec, src/Solver.cpp:648-656): last reference dimension first, as a
// tensor product. A CTA takes tiles of EPB elements; stage m (m = 1..nd) interpolates along
// dimension nd - m the (nvert >> (m-1)) x RS^(m-1) values of the previous stage to
// (nvert >> m) x RS^m, in shared memory, so each point's value comes out of the same operations
// as interpolating its nvert vertex values one point at a time, with the partial results shared
// (312 instead of 1512 interpolations per element at row size 6 in 3D). R as in k_av_uncert.
template <int ND, int RS, typename R>
__global__ void __launch_bounds__(Shape<ND, RS>::threads)
k_av_interp(double* elem, const int* vert_id, int n_elem, AvTab<RS, R> tab, const double* vmax)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nv = S::nv, nvert = S::nvert, EPB = S::epb;
  __shared__ R s_buf[2][EPB*nq];
  __shared__ R s_node[RS];
  if (threadIdx.x == 0) {   // constant indices, as in k_av_uncert; the tile loop's barrier follows
    #pragma unroll
    for (int i = 0; i < RS; ++i) s_node[i] = tab.node[i];
  }
  const int n_tiles = (n_elem + EPB - 1)/EPB;
  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int e0 = tile*EPB;
    __syncthreads();   // the previous tile's last stage is read
    for (int i = threadIdx.x; i < EPB*nvert; i += blockDim.x)
      s_buf[0][i] = e0 + i/nvert < n_elem ? to_R<R>(vmax[vert_id[(size_t)e0*nvert + i]]) : R(0);
    #pragma unroll
    for (int m = 1; m <= ND; ++m) {
      __syncthreads();
      const int sub = ipow(RS, m - 1);
      const int n_in = (nvert >> (m - 1))*sub, n_out = (nvert >> m)*sub*RS;
      const R* in = s_buf[(m - 1)%2];
      R* out = s_buf[m%2];
      for (int t = threadIdx.x; t < EPB*n_out; t += blockDim.x) {
        const int le = t/n_out, o = t%n_out;
        const int i = o/(sub*RS), p = o%(sub*RS);
        const int rest = p%sub;
        const R x = s_node[p/sub];
        const R* a = in + le*n_in + 2*i*sub + rest;
        const R v = (R(1) - x)*a[0] + x*a[sub];
        if (m < ND) out[le*n_out + o] = v;
        else if (e0 + le < n_elem) elem[(size_t)(e0 + le)*(nv + 3)*nq + (nv + 2)*nq + p] = double(v);
      }
    }
  }
}

// ------------------------------------------------------------------- residual norm
// integral_field(Pow(Physical_residual, 2)) (src/Solver.cpp:1113-1131): per-CTA partial
// sums in a fixed order, then one CTA sums the partials in order (deterministic).
template <int ND, int RS, typename FaceT>
__global__ void __launch_bounds__(256) k_residual_partial(Dev<FaceT> m, Tab<RS> tab, double* partials)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nv = S::nv;
  double acc[nv];
  for (int v = 0; v < nv; ++v) acc[v] = 0.;
  const long total = (long)m.n_elem*nq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int e = int(t/nq), q = int(t%nq);
    double w = 1.;
    for (int d = 0; d < ND; ++d) w *= tab.weight[(q/ipow(RS, ND - 1 - d))%RS];
    double vol = 1.;
    for (int d = 0; d < ND; ++d) vol *= m.nom_size[e];
    const double* st = m.elem + (size_t)e*(nv + 3)*nq;
    const FaceT* rc = m.rcache + (size_t)e*nv*nq;
    const double jd = e >= m.n_car ? m.jac[((size_t)(e - m.n_car)*(ND*ND + 1) + ND*ND)*nq + q] : 1.;
    const double tss = st[nv*nq + q];
    for (int v = 0; v < nv; ++v) {
      double r = double(rc[v*nq + q])/tss;
      acc[v] += w*vol*(r*r)*jd;
    }
  }
  __shared__ double s_acc[256][nv];
  for (int v = 0; v < nv; ++v) s_acc[threadIdx.x][v] = acc[v];
  __syncthreads();
  for (int half = blockDim.x/2; half > 0; half >>= 1) {
    if ((int)threadIdx.x < half) for (int v = 0; v < nv; ++v) s_acc[threadIdx.x][v] += s_acc[threadIdx.x + half][v];
    __syncthreads();
  }
  if (threadIdx.x == 0) for (int v = 0; v < nv; ++v) partials[blockIdx.x*nv + v] = s_acc[0][v];
}

// Residual norms of independent element segments (one solve each): CTA i reduces segment i
// alone, in a fixed order, so its result is the same whatever else the arena holds.
template <int ND, int RS, typename FaceT>
__global__ void __launch_bounds__(256) k_segment_residual(Dev<FaceT> m, Tab<RS> tab, const int* seg_begin,
                                                          const int* seg_count, double* out)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nv = S::nv;
  const int e_first = seg_begin[blockIdx.x];
  const long total = (long)seg_count[blockIdx.x]*nq;
  double acc[nv];
  for (int v = 0; v < nv; ++v) acc[v] = 0.;
  for (long t = threadIdx.x; t < total; t += blockDim.x) {
    const int e = e_first + int(t/nq), q = int(t%nq);
    double w = 1.;
    for (int d = 0; d < ND; ++d) w *= tab.weight[(q/ipow(RS, ND - 1 - d))%RS];
    double vol = 1.;
    for (int d = 0; d < ND; ++d) vol *= m.nom_size[e];
    const double* st = m.elem + (size_t)e*(nv + 3)*nq;
    const FaceT* rc = m.rcache + (size_t)e*nv*nq;
    const double jd = e >= m.n_car ? m.jac[((size_t)(e - m.n_car)*(ND*ND + 1) + ND*ND)*nq + q] : 1.;
    const double tss = st[nv*nq + q];
    for (int v = 0; v < nv; ++v) {
      double r = double(rc[v*nq + q])/tss;
      acc[v] += w*vol*(r*r)*jd;
    }
  }
  __shared__ double s_acc[256][nv];
  for (int v = 0; v < nv; ++v) s_acc[threadIdx.x][v] = acc[v];
  __syncthreads();
  for (int half = blockDim.x/2; half > 0; half >>= 1) {
    if ((int)threadIdx.x < half) for (int v = 0; v < nv; ++v) s_acc[threadIdx.x][v] += s_acc[threadIdx.x + half][v];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double mom = 0.;
    for (int d = 0; d < ND; ++d) mom += s_acc[0][d];
    out[3*blockIdx.x] = sqrt(mom);
    out[3*blockIdx.x + 1] = sqrt(s_acc[0][ND]);
    out[3*blockIdx.x + 2] = sqrt(s_acc[0][ND + 1]);
  }
}

template <int NV>
__global__ void k_residual_final(const double* partials, int n_part, double* out)
{
  if (threadIdx.x != 0) return;
  double acc[NV];
  for (int v = 0; v < NV; ++v) acc[v] = 0.;
  for (int i = 0; i < n_part; ++i) for (int v = 0; v < NV; ++v) acc[v] += partials[i*NV + v];
  double mom = 0.;
  for (int d = 0; d < NV - 2; ++d) mom += acc[d];
  out[0] = sqrt(mom);
  out[1] = sqrt(acc[NV - 2]);
  out[2] = sqrt(acc[NV - 1]);
}

} // namespace hx
