// hexed_oracle.cpp -- TEST INFRASTRUCTURE ONLY: the CPU oracle of the DG hot path.
//
// A plain C++ (no Eigen) restatement of hexed's OpenMP kernels, operating in place on
// the flat mesh arena declared in include/hexed_gpu.h. It is the checker the parity
// tests hold the CUDA library against and the CPU baseline the benchmark times; the
// product (hexed_gb300/csrc) never includes or links it.
//
// Each function follows the reference operation by operation so that its rounding
// matches the reference's own arithmetic; the file:line it restates is cited on it.
// Deliberate differences, all at the roundoff level:
//  * small matrix products and norms sum in ascending index order (Eigen may use
//    SIMD partial sums);
//  * the 3x3 characteristic system of the Riemann-invariant BC is solved by Gaussian
//    elimination with partial pivoting instead of Eigen's column-pivoted QR (the
//    solutions agree to roundoff whenever pressure > 0, i.e. the system is regular);
//  * the build uses -ffp-contract=off so results do not depend on the host ISA.
// Parity of this restatement with the reference is pinned by the reference's own
// tests (analytic and property checks, restated under tests/) and by the basis
// tables generated with the reference's generator (tests/golden/).
#include <cmath>
#include <cstring>
#include <cstdint>
#include <algorithm>
#include <limits>
#include <vector>
#include <type_traits>
#include <omp.h>
#include "../include/hexed_gpu.h"
#include "../hexed_gb300/csrc/basis_tables.h"

// Parameters of Solver::update_art_visc_smoothness (src/Solver.cpp:457-582) and
// Solver::diffuse_art_visc (src/Solver.cpp:428-455); the reference's defaults
// (src/Solver.cpp:154-163) in brackets.
struct oracle_sav_params {
  double advect_length;      // the `advect_length` argument (Case: art_visc_width)
  int advect_iters;          // av_advect_iters [1]
  int diff_iters;            // av_diff_iters [1]
  int n_cheby;               // n_cheby_av [1]
  int av_row_size;           // av_rs: degree + 1 of the projected Legendre mode [row_size]
  double advect_safety;      // av_advect_max_safety [0.7]
  double diff_safety;        // av_diff_max_safety [0.7]
  double diff_ratio;         // av_diff_ratio [0.3]
  double visc_mult;          // av_visc_mult [100]
  double unscaled_max;       // av_unscaled_max [5]
  double freestream_mass;    // freestream{n_dim}
  double freestream_energy;  // freestream{n_dim + 1}
};

namespace {

constexpr double heat_rat = 1.4;                 // include/pde.hpp:51
constexpr double specific_gas_air = 287.05287;   // include/constants.hpp:44

constexpr int ipow(int b, int e) { int r = 1; for (int i = 0; i < e; ++i) r *= b; return r; }

struct Tables {
  const double* node; const double* weight; const double* diff; const double* bound;
  const double* filter; const double* prolong; const double* restrict_; const double* ortho;
  double max_cfl, min_eig_diffusion, step_ratio;
};

Tables tables(int rs)
{
  using namespace hexed_tables;
  switch (rs) {
#define HEXED_T(n) case n: return {node##n, weight##n, diff_mat##n, boundary##n, filter##n, prolong##n, restrict_##n, orthogonal##n, max_cfl##n, min_eig_diffusion##n, step_ratio};
    HEXED_T(2) HEXED_T(3) HEXED_T(4) HEXED_T(5) HEXED_T(6) HEXED_T(7) HEXED_T(8)
#undef HEXED_T
  }
  return {};
}

// Transport_model::coefficient (include/Transport_model.hpp:35-38)
inline double transport_coef(const hexed_transport& t, double sqrt_temp)
{
  double r = sqrt_temp/std::sqrt(t.ref_temp);
  double p3 = 1.; p3 *= r; p3 *= r; p3 *= r;   // math::pow(x, 3), include/math.hpp:30-36
  return t.const_val + t.ref_val*p3*(t.ref_temp + t.temp_offset)/(sqrt_temp*sqrt_temp + t.temp_offset);
}

template <int ND, int RS>
struct K
{
  static constexpr int n_dim = ND, row_size = RS;
  static constexpr int nq = ipow(RS, ND);
  static constexpr int nfq = nq/RS;
  static constexpr int nv = ND + 2;
  static constexpr int nvert = 1 << ND;
  static constexpr int n_slot_dof = 2*nv*nfq;

  const hexed_mesh_desc& m;
  Tables t;
  double lift[RS][2];   // Derivative::lift (include/Derivative.hpp:22-28)
  // true while Solver::fix_admissibility diffuses the state: the viscous kernels, Max_dt and
  // the boundary conditions then compute pde::Fix_therm_admis (include/pde.hpp:437-493)
  mutable bool fta = false;
  explicit K(const hexed_mesh_desc& mesh) : m{mesh}, t{tables(RS)}
  {
    for (int i = 0; i < RS; ++i) {
      double inv_w = 1./t.weight[i];
      lift[i][0] = -(inv_w*t.bound[0*RS + i]);
      lift[i][1] = inv_w*t.bound[1*RS + i];
    }
  }

  int n_elem() const { return m.n_car_elem + m.n_def_elem; }
  double* elem(int e) const { return m.elem + (size_t)e*(nv + 3)*nq; }
  double* rcache(int e) const { return m.rcache + (size_t)e*nv*nq; }
  double* slot(int s, bool ldg) const { return m.face + (size_t)s*n_slot_dof + ldg*nv*nfq; }
  double* face(int e, int i_face, bool ldg) const { return slot(e*2*ND + i_face, ldg); }

  // Row_index (include/Row_index.hpp:14-64)
  static int row_stride(int i_dim) { return ipow(RS, ND - 1 - i_dim); }
  static int row_qpoint(int i_dim, int i_fq, int i_node)
  {
    int stride = row_stride(i_dim);
    return (i_fq/stride)*stride*RS + i_fq%stride + i_node*stride;
  }

  // Derivative::operator() (include/Derivative.hpp:50-55): diff*f + lift*(fb - B*f)
  void derivative(const double* f, const double* fb, double* out) const
  {
    double bf[2];
    for (int s = 0; s < 2; ++s) {
      double acc = 0.;
      for (int j = 0; j < RS; ++j) acc += t.bound[s*RS + j]*f[j];
      bf[s] = fb[s] - acc;
    }
    for (int i = 0; i < RS; ++i) {
      double d = 0.;
      for (int j = 0; j < RS; ++j) d += t.diff[i*RS + j]*f[j];
      double l = 0.;
      l += lift[i][0]*bf[0];
      l += lift[i][1]*bf[1];
      out[i] = d + l;
    }
  }
  void derivative_interior(const double* f, double* out) const // Derivative.hpp:56-60
  {
    for (int i = 0; i < RS; ++i) {
      double d = 0.;
      for (int j = 0; j < RS; ++j) d += t.diff[i*RS + j]*f[j];
      out[i] = d;
    }
  }

  // Spatial::Write_face::operator() (include/Spatial.hpp:41-57)
  void write_face_elem(const double* state, double* const* faces) const
  {
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        for (int v = 0; v < nv; ++v) {
          for (int s = 0; s < 2; ++s) {
            double acc = 0.;
            for (int i = 0; i < RS; ++i) acc += t.bound[s*RS + i]*state[v*nq + row_qpoint(d, i_fq, i)];
            faces[2*d + s][v*nfq + i_fq] = acc;
          }
        }
      }
    }
  }

  void write_face() const // Write_face over all elements (Spatial.hpp:60-70)
  {
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) {
      double* faces[6];
      for (int i = 0; i < 2*ND; ++i) faces[i] = face(e, i, false);
      write_face_elem(elem(e), faces);
    }
  }

  // ---------------------------------------------------------------- PDE pieces
  // Navier_stokes::Pde::Computation::compute_scalars_conv (include/pde.hpp:97-104)
  struct Conv { double mass, kin_ener, pressure; };
  static Conv scalars_conv(const double* s)
  {
    Conv c;
    c.mass = s[ND];
    c.kin_ener = 0;
    for (int d = 0; d < ND; ++d) c.kin_ener += s[d]*s[d];
    c.kin_ener *= .5/c.mass;
    c.pressure = (heat_rat - 1.)*(s[ND + 1] - c.kin_ener);
    return c;
  }
  // compute_flux_conv for one flux direction given by column `n` (pde.hpp:108-122)
  static void flux_conv(const double* s, const Conv& c, const double* n, double* f)
  {
    f[ND] = 0;
    for (int j = 0; j < ND; ++j) f[ND] += s[j]*n[j];
    double vol_flux = f[ND]/c.mass;
    f[ND + 1] = (s[ND + 1] + c.pressure)*vol_flux;
    for (int j = 0; j < ND; ++j) f[j] = s[j]*vol_flux + c.pressure*n[j];
  }
  // compute_char_speed (pde.hpp:161-166)
  static double char_speed(const double* s)
  {
    double sound_speed = std::sqrt(heat_rat*(heat_rat - 1)*s[ND + 1]/s[ND]);
    double sq = 0.;
    for (int d = 0; d < ND; ++d) sq += s[d]*s[d];
    return sound_speed + std::sqrt(sq)/s[ND];
  }
  struct Diff { double bulk_av, laplacian_av, sqrt_temp, mu, k, energy_cond; };
  // compute_scalars_diff (pde.hpp:130-138); s has nv + 2 entries (bulk, Laplacian AV)
  static Diff scalars_diff(const double* s, const Conv& c, const hexed_transport& visc, const hexed_transport& cond)
  {
    Diff d;
    d.bulk_av = std::abs(s[ND + 2]);
    d.laplacian_av = std::abs(s[ND + 3]);
    d.sqrt_temp = std::sqrt(std::max((s[ND + 1] - c.kin_ener)/c.mass, 0.)*(heat_rat - 1)/specific_gas_air);
    d.mu = transport_coef(visc, d.sqrt_temp);
    d.k = transport_coef(cond, d.sqrt_temp);
    d.energy_cond = d.k*(heat_rat - 1)/specific_gas_air;
    return d;
  }
  // compute_flux_diff (pde.hpp:142-158). g[nv][ND] gradient, nrm[ND][ND] (row = physical
  // dim, column = reference dim), out fd[nv][ND].
  static void flux_diff(const double* s, const Conv& c, const Diff& df, const double (*g)[ND],
                        const double (*nrm)[ND], bool identity, double (*out)[ND])
  {
    double mass = c.mass;
    double veloc[ND];
    for (int i = 0; i < ND; ++i) veloc[i] = s[i]/mass;
    double vg[ND][ND];
    for (int i = 0; i < ND; ++i) for (int j = 0; j < ND; ++j) vg[i][j] = (g[i][j] - veloc[i]*g[ND][j])/mass;
    double trace = 0.;
    for (int i = 0; i < ND; ++i) trace += vg[i][i];
    double bulk_term = (df.bulk_av*mass - 2./3.*df.mu)*trace;
    double stress[ND][ND];
    for (int i = 0; i < ND; ++i) for (int j = 0; j < ND; ++j)
      stress[i][j] = df.mu*(vg[i][j] + vg[j][i]) + bulk_term*(i == j ? 1. : 0.);
    double fd[ND + 2][ND];
    for (int v = 0; v < ND + 2; ++v) for (int j = 0; j < ND; ++j) fd[v][j] = -df.laplacian_av*g[v][j];
    for (int i = 0; i < ND; ++i) for (int j = 0; j < ND; ++j) fd[i][j] -= stress[i][j];
    double coef = -s[ND + 1]/mass/mass;
    for (int j = 0; j < ND; ++j) {
      double vvg = 0.;
      for (int i = 0; i < ND; ++i) vvg += veloc[i]*vg[i][j];
      double ieg = coef*g[ND][j] + g[ND + 1][j]/mass - vvg;
      double vs = 0.;
      for (int i = 0; i < ND; ++i) vs += veloc[i]*stress[i][j];
      fd[ND + 1][j] -= vs + df.energy_cond*ieg;
    }
    for (int v = 0; v < ND + 2; ++v) {
      for (int i = 0; i < ND; ++i) {
        if (identity) { out[v][i] = fd[v][i]; continue; }
        double acc = 0.;
        for (int j = 0; j < ND; ++j) acc += fd[v][j]*nrm[j][i];
        out[v][i] = acc;
      }
    }
  }

  // ---------------------------------------------------------------- Face_permutation
  // Index in face-1 storage of the value that lands at face-0 qpoint q after
  // Face_permutation::match_faces (transpose then flip; include/Spatial.hpp:85-129).
  static int perm_index(int dir_packed, int q)
  {
    int i_dim0 = dir_packed & 3, i_dim1 = (dir_packed >> 2) & 3;
    bool s0 = (dir_packed >> 4) & 1, s1 = (dir_packed >> 5) & 1;
    bool flip_n0 = (s0 == 0), flip_n1 = (s1 == 1);           // Connection_direction::flip_normal
    bool flip_tan = (i_dim0 != i_dim1) && (flip_n0 == flip_n1);
    bool transpose = ((i_dim0 == 0) && (i_dim1 == 2)) || ((i_dim0 == 2) && (i_dim1 == 0));
    if (ND == 3) {
      // column-major rs x rs map: (r, c) at r + c*rs
      int r = q%RS, c = q/RS;
      if (flip_tan) {
        bool colwise = (i_dim0 > 3 - i_dim0 - i_dim1) != transpose;
        if (colwise) r = RS - 1 - r; else c = RS - 1 - c;
      }
      int idx = r + c*RS;
      if (transpose) idx = (idx%RS)*RS + idx/RS;
      return idx;
    } else if (ND == 2) {
      return flip_tan ? RS - 1 - q : q;
    }
    return q;
  }

  // ---------------------------------------------------------------- Neighbor
  // Spatial::Neighbor::operator() (include/Spatial.hpp:613-705) for one connection.
  // `nrml` is null for Cartesian connections (normal = unit vector along i_dim0).
  void neighbor_con(int slot0, int slot1, int dir, const double* nrml, bool viscous) const
  {
    int i_dim0 = dir & 3;
    int sign[2] = {1, 1};
    bool deformed = nrml != nullptr;
    if (deformed) {
      bool s0 = (dir >> 4) & 1, s1 = (dir >> 5) & 1;
      sign[0] = 1 - 2*(s0 == 0);
      sign[1] = 1 - 2*(s1 == 1);
    }
    double* f0 = slot(slot0, false);
    double* f1 = slot(slot1, false);
    double* l0 = slot(slot0, true);
    double* l1 = slot(slot1, true);
    double out0[nv*nfq], out1[nv*nfq];
    double avg0[nv*nfq], avg1[nv*nfq];
    for (int q = 0; q < nfq; ++q) {
      int q1 = deformed ? perm_index(dir, q) : q;
      double u[2][nv + 2];
      for (int v = 0; v < nv; ++v) { u[0][v] = f0[v*nfq + q]; u[1][v] = f1[v*nfq + q1]; }
      if (viscous) {
        for (int v = 0; v < nv; ++v) {
          double avg = .5*(u[0][v] + u[1][v]);
          avg0[v*nfq + q] = avg;
          avg1[v*nfq + q1] = avg;
        }
      }
      if (fta) continue;   // Fix_therm_admis has no convection (Spatial.hpp:655-686)
      double n[ND];
      if (deformed) for (int d = 0; d < ND; ++d) n[d] = sign[0]*nrml[d*nfq + q];
      else for (int d = 0; d < ND; ++d) n[d] = (d == i_dim0) ? 1. : 0.;
      double fl[2][nv], cs[2];
      for (int side = 0; side < 2; ++side) {
        Conv c = scalars_conv(u[side]);
        flux_conv(u[side], c, n, fl[side]);
        cs[side] = char_speed(u[side]);
      }
      double nn = 0.;
      for (int d = 0; d < ND; ++d) nn += n[d]*n[d];
      double mult = std::max(cs[0], cs[1])*std::sqrt(nn);
      for (int v = 0; v < nv; ++v) {
        double flux = .5*(fl[0][v] + fl[1][v] + mult*(u[0][v] - u[1][v]));
        out0[v*nfq + q] = sign[0]*flux;
        out1[v*nfq + q1] = sign[1]*flux;
      }
    }
    if (!fta) {
      std::memcpy(f0, out0, sizeof(out0));
      std::memcpy(f1, out1, sizeof(out1));
    }
    if (viscous) {
      std::memcpy(l0, avg0, sizeof(avg0));
      std::memcpy(l1, avg1, sizeof(avg1));
    }
  }

  void neighbor(bool viscous) const
  {
    #pragma omp parallel for
    for (int i = 0; i < m.n_car_con; ++i) {
      const int* c = m.car_con + 3*i;
      neighbor_con(c[0], c[1], c[2] | (c[2] << 2) | (1 << 4), nullptr, viscous);
    }
    #pragma omp parallel for
    for (int i = 0; i < m.n_def_con; ++i) {
      const int* c = m.def_con + 3*i;
      neighbor_con(c[0], c[1], c[2], m.def_con_nrml + (size_t)i*ND*nfq, viscous);
    }
    // boundary connections are deformed connections with direction {{d,d},{ifs,!ifs}}
    // (include/connection.hpp:378, src/Accessible_mesh.cpp:136-146)
    #pragma omp parallel for
    for (int i = 0; i < m.n_bc_con; ++i) {
      const int* c = m.bc_con + 4*i;
      int d = c[2] & 3, ifs = (c[2] >> 2) & 1;
      int dir = d | (d << 2) | (ifs << 4) | ((!ifs) << 5);
      neighbor_con(c[0], c[1], dir, m.bc_nrml + (size_t)i*ND*nfq, viscous);
    }
  }

  // Spatial::Neighbor_reconcile (include/Spatial.hpp:716-759) for one connection
  void reconcile_con(int slot0, int slot1, int dir, bool deformed) const
  {
    int sign[2] = {1, 1};
    if (deformed) {
      bool s0 = (dir >> 4) & 1, s1 = (dir >> 5) & 1;
      sign[0] = 1 - 2*(s0 == 0);
      sign[1] = 1 - 2*(s1 == 1);
    }
    double* l0 = slot(slot0, true);
    double* l1 = slot(slot1, true);
    double out0[nv*nfq], out1[nv*nfq];
    for (int q = 0; q < nfq; ++q) {
      int q1 = deformed ? perm_index(dir, q) : q;
      for (int v = 0; v < nv; ++v) {
        double a = l0[v*nfq + q], b = l1[v*nfq + q1];
        double avg = 0;
        avg += .5*sign[0]*a;
        avg += .5*sign[1]*b;
        out0[v*nfq + q] = sign[0]*avg - a;
        out1[v*nfq + q1] = sign[1]*avg - b;
      }
    }
    std::memcpy(l0, out0, sizeof(out0));
    std::memcpy(l1, out1, sizeof(out1));
  }

  void neighbor_reconcile() const
  {
    #pragma omp parallel for
    for (int i = 0; i < m.n_car_con; ++i) {
      const int* c = m.car_con + 3*i;
      reconcile_con(c[0], c[1], 0, false);
    }
    #pragma omp parallel for
    for (int i = 0; i < m.n_def_con; ++i) {
      const int* c = m.def_con + 3*i;
      reconcile_con(c[0], c[1], c[2], true);
    }
    #pragma omp parallel for
    for (int i = 0; i < m.n_bc_con; ++i) {
      const int* c = m.bc_con + 4*i;
      int d = c[2] & 3, ifs = (c[2] >> 2) & 1;
      reconcile_con(c[0], c[1], d | (d << 2) | (ifs << 4) | ((!ifs) << 5), true);
    }
  }

  // ---------------------------------------------------------------- Local
  // Spatial::Local::operator() (include/Spatial.hpp:326-509) for one element.
  void local_elem(int e, bool deformed, bool viscous, double update_coef, int stage,
                  bool compute_residual, bool use_filter,
                  const hexed_transport& visc, const hexed_transport& cond) const
  {
    double* state = elem(e);
    double* tss = state + nv*nq;
    double d_pos = m.nom_size[e];
    double* faces[6];
    double* visc_faces[6];
    for (int i = 0; i < 2*ND; ++i) { faces[i] = face(e, i, false); visc_faces[i] = face(e, i, true); }
    const double* nrml = nullptr;
    const double* det = nullptr;
    const double* face_nrml[6] = {};
    if (deformed) {
      int ed = e - m.n_car_elem;
      nrml = m.jac + (size_t)ed*(ND*ND + 1)*nq;
      det = nrml + ND*ND*nq;
      for (int i = 0; i < 2*ND; ++i) face_nrml[i] = m.face_nrml + ((size_t)ed*2*ND + i)*ND*nfq;
    }
    static thread_local std::vector<double> buf;
    buf.assign((size_t)(2*nv*nq + ND*nv*nq + ND*nv*nq), 0.);
    double (*time_rate)[nv][nq] = reinterpret_cast<double (*)[nv][nq]>(buf.data());
    double (*visc_storage)[nv][nq] = reinterpret_cast<double (*)[nv][nq]>(buf.data() + 2*nv*nq);
    double (*flux)[nv][nq] = reinterpret_cast<double (*)[nv][nq]>(buf.data() + 2*nv*nq + ND*nv*nq);

    if (viscous) {
      // gradient times Jacobian determinant (Spatial.hpp:371-402)
      for (int v = 0; v < nv; ++v) for (int q = 0; q < nq; ++q) time_rate[0][v][q] = state[v*nq + q];
      for (int d = 0; d < ND; ++d) {
        for (int i_fq = 0; i_fq < nfq; ++i_fq) {
          double row_r[nv][RS], fs[nv][2];
          for (int v = 0; v < nv; ++v) {
            for (int i = 0; i < RS; ++i) row_r[v][i] = time_rate[0][v][row_qpoint(d, i_fq, i)];
            for (int s = 0; s < 2; ++s) fs[v][s] = visc_faces[2*d + s][v*nfq + i_fq];
          }
          if (deformed) {
            for (int j = 0; j < ND; ++j) {
              double row_n[RS], face_n[2];
              for (int i = 0; i < RS; ++i) row_n[i] = nrml[(d*ND + j)*nq + row_qpoint(d, i_fq, i)];
              for (int s = 0; s < 2; ++s) face_n[s] = face_nrml[2*d + s][j*nfq + i_fq];
              for (int v = 0; v < nv; ++v) {
                double row[RS], bound[2], der[RS];
                for (int i = 0; i < RS; ++i) row[i] = row_n[i]*row_r[v][i];
                for (int s = 0; s < 2; ++s) bound[s] = face_n[s]*fs[v][s];
                derivative(row, bound, der);
                for (int i = 0; i < RS; ++i) {
                  double& x = visc_storage[j][v][row_qpoint(d, i_fq, i)];
                  x = 1.*x + der[i]/d_pos;
                }
              }
            }
          } else {
            for (int v = 0; v < nv; ++v) {
              double der[RS];
              derivative(row_r[v], fs[v], der);
              for (int i = 0; i < RS; ++i) {
                double& x = visc_storage[d][v][row_qpoint(d, i_fq, i)];
                x = 0*x + der[i]/d_pos;
              }
            }
          }
        }
      }
      for (int v = 0; v < nv; ++v) for (int q = 0; q < nq; ++q) { time_rate[0][v][q] = 0; time_rate[1][v][q] = 0; }
    }

    // flux (Spatial.hpp:405-442)
    for (int q = 0; q < nq; ++q) {
      double s[nv + 2];
      for (int v = 0; v < nv; ++v) s[v] = state[v*nq + q];
      s[nv] = state[(nv + 1)*nq + q];
      s[nv + 1] = state[(nv + 2)*nq + q];
      double nmat[ND][ND]; // nmat[j][i] = comp.normal(j, i)
      for (int i = 0; i < ND; ++i) for (int j = 0; j < ND; ++j)
        nmat[j][i] = deformed ? nrml[(i*ND + j)*nq + q] : (i == j ? 1. : 0.);
      Conv c = scalars_conv(s);
      if (!fta) {
        for (int i = 0; i < ND; ++i) {
          double col[ND], f[nv];
          for (int j = 0; j < ND; ++j) col[j] = nmat[j][i];
          flux_conv(s, c, col, f);
          for (int v = 0; v < nv; ++v) flux[i][v][q] = f[v];
        }
      }
      if (viscous) {
        double g[nv][ND];
        for (int d = 0; d < ND; ++d) for (int v = 0; v < nv; ++v) g[v][d] = visc_storage[d][v][q];
        if (deformed) for (int v = 0; v < nv; ++v) for (int d = 0; d < ND; ++d) g[v][d] /= det[q];
        double fd[nv][ND];
        if (fta) {
          // Fix_therm_admis::compute_flux_diff (include/pde.hpp:481-485): -gradient*normal
          for (int v = 0; v < nv; ++v) for (int i = 0; i < ND; ++i) {
            double acc = 0.;
            for (int j = 0; j < ND; ++j) acc += -g[v][j]*nmat[j][i];
            fd[v][i] = acc;
          }
        } else {
          Diff df = scalars_diff(s, c, visc, cond);
          flux_diff(s, c, df, g, nmat, !deformed, fd);
        }
        for (int d = 0; d < ND; ++d) for (int v = 0; v < nv; ++v) visc_storage[d][v][q] = fd[v][d];
      }
    }

    // residual (Spatial.hpp:445-470)
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        for (int v = 0; v < nv; ++v) {
          double row_f[RS], face_f[2], der[RS];
          if (!fta) {
            for (int i = 0; i < RS; ++i) row_f[i] = flux[d][v][row_qpoint(d, i_fq, i)];
            for (int s = 0; s < 2; ++s) face_f[s] = faces[2*d + s][v*nfq + i_fq];
            derivative(row_f, face_f, der);
            for (int i = 0; i < RS; ++i) {
              double& x = time_rate[0][v][row_qpoint(d, i_fq, i)];
              x = 1.*x + -der[i];
            }
          }
          if (viscous) {
            for (int i = 0; i < RS; ++i) row_f[i] = visc_storage[d][v][row_qpoint(d, i_fq, i)];
            for (int s = 0; s < 2; ++s) {
              double acc = 0.;
              for (int i = 0; i < RS; ++i) acc += t.bound[s*RS + i]*row_f[i];
              visc_faces[2*d + s][v*nfq + i_fq] = acc;
            }
            derivative_interior(row_f, der);
            for (int i = 0; i < RS; ++i) {
              double& x = time_rate[1][v][row_qpoint(d, i_fq, i)];
              x = 1.*x + -der[i];
            }
          }
        }
      }
    }

    // modal filter (Spatial.hpp:473-481)
    if (use_filter) {
      for (int d = 0; d < ND; ++d) {
        for (int i_fq = 0; i_fq < nfq; ++i_fq) {
          for (int k = 0; k < 2; ++k) for (int v = 0; v < nv; ++v) {
            double row[RS];
            for (int i = 0; i < RS; ++i) row[i] = time_rate[k][v][row_qpoint(d, i_fq, i)];
            for (int i = 0; i < RS; ++i) {
              double acc = 0.;
              for (int j = 0; j < RS; ++j) acc += t.filter[i*RS + j]*row[j];
              double& x = time_rate[k][v][row_qpoint(d, i_fq, i)];
              x = 0.*x + acc;
            }
          }
        }
      }
    }

    // update (Spatial.hpp:484-503)
    double* ref_state = rcache(e);
    for (int q = 0; q < nq; ++q) {
      double update[nv] = {};
      double mult = update_coef*tss[q]/d_pos;
      if (deformed) mult /= det[q];
      for (int v = 0; v < nv; ++v) {
        double u = time_rate[0][v][q];
        if (stage) {
          u -= ref_state[v*nq + q];
        } else {
          if (!fta) ref_state[v*nq + q] = u;   // Pde::has_convection
          if (viscous) u += time_rate[1][v][q];
        }
        u *= mult;
        if (compute_residual) ref_state[v*nq + q] = u;
        else update[v] = u;
      }
      for (int v = 0; v < nv; ++v) state[v*nq + q] += update[v];
    }
    if (!viscous) write_face_elem(state, faces);
  }

  void local(bool viscous, double dt, int stage, bool compute_residual, bool use_filter,
             const hexed_transport& visc, const hexed_transport& cond) const
  {
    double update_coef = stage ? dt*t.step_ratio : dt;
    #pragma omp parallel for
    for (int e = 0; e < m.n_car_elem; ++e)
      local_elem(e, false, viscous, update_coef, stage, compute_residual, use_filter, visc, cond);
    #pragma omp parallel for
    for (int e = m.n_car_elem; e < n_elem(); ++e)
      local_elem(e, true, viscous, update_coef, stage, compute_residual, use_filter, visc, cond);
  }

  // Spatial::Reconcile_ldg_flux (include/Spatial.hpp:543-594)
  void reconcile_ldg_elem(int e, bool deformed, double dt, bool compute_residual, bool use_filter) const
  {
    double* state = elem(e);
    double* tss = state + nv*nq;
    double d_pos = m.nom_size[e];
    const double* det = nullptr;
    if (deformed) det = m.jac + (size_t)(e - m.n_car_elem)*(ND*ND + 1)*nq + ND*ND*nq;
    double time_rate[nv][nq];
    for (int v = 0; v < nv; ++v) for (int q = 0; q < nq; ++q) time_rate[v][q] = 0.;
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        for (int v = 0; v < nv; ++v) {
          double b0 = face(e, 2*d, true)[v*nfq + i_fq];
          double b1 = face(e, 2*d + 1, true)[v*nfq + i_fq];
          for (int i = 0; i < RS; ++i) {
            double l = 0.;
            l += lift[i][0]*b0;
            l += lift[i][1]*b1;
            double& x = time_rate[v][row_qpoint(d, i_fq, i)];
            x = 1.*x + -l;
          }
        }
      }
    }
    if (use_filter) {
      for (int d = 0; d < ND; ++d) for (int i_fq = 0; i_fq < nfq; ++i_fq) for (int v = 0; v < nv; ++v) {
        double row[RS];
        for (int i = 0; i < RS; ++i) row[i] = time_rate[v][row_qpoint(d, i_fq, i)];
        for (int i = 0; i < RS; ++i) {
          double acc = 0.;
          for (int j = 0; j < RS; ++j) acc += t.filter[i*RS + j]*row[j];
          double& x = time_rate[v][row_qpoint(d, i_fq, i)];
          x = 0.*x + acc;
        }
      }
    }
    double* to_update = compute_residual ? rcache(e) : state;
    for (int q = 0; q < nq; ++q) {
      double mult = dt*tss[q]/d_pos;
      if (deformed) mult /= det[q];
      for (int v = 0; v < nv; ++v) to_update[v*nq + q] += time_rate[v][q]*mult;
    }
    double* faces[6];
    for (int i = 0; i < 2*ND; ++i) faces[i] = face(e, i, false);
    write_face_elem(state, faces);
  }

  void reconcile_ldg_flux(double dt, bool compute_residual, bool use_filter) const
  {
    #pragma omp parallel for
    for (int e = 0; e < m.n_car_elem; ++e) reconcile_ldg_elem(e, false, dt, compute_residual, use_filter);
    #pragma omp parallel for
    for (int e = m.n_car_elem; e < n_elem(); ++e) reconcile_ldg_elem(e, true, dt, compute_residual, use_filter);
  }

  // ---------------------------------------------------------------- hanging faces
  // Spatial::Prolong_refined / Restrict_refined (include/Spatial.hpp:153-206, 230-285)
  void refine(bool prolong, bool scale, bool offset) const
  {
    refine_slots(m.face, n_slot_dof, nv, prolong, scale, offset);
  }

  // the same over face slots of `slot_stride` doubles from `base` and the first n_var face
  // variables (the Pde's n_extrap, Spatial.hpp:141, 218); the LDG half starts at nv*nfq
  void refine_slots(double* base, size_t slot_stride, int n_var, bool prolong, bool scale, bool offset) const
  {
    const int n_face = 1 << (ND - 1);
    #pragma omp parallel for
    for (int i_ref = 0; i_ref < m.n_ref_face; ++i_ref) {
      const int* rf = m.ref_face + 7*i_ref;
      bool str[2] = {rf[5] != 0, rf[6] != 0};
      double* coarse = base + (size_t)rf[0]*slot_stride + offset*nv*nfq;
      if (!prolong) for (int i = 0; i < n_var*nfq; ++i) coarse[i] = 0.;
      int nf = n_face;
      for (int d = 0; d < ND - 1; ++d) nf /= 1 + str[d];
      for (int i_face = 0; i_face < nf; ++i_face) {
        double* fine = base + (size_t)rf[1 + i_face]*slot_stride + offset*nv*nfq;
        for (int v = 0; v < n_var; ++v) {
          double* var_face = fine + v*nfq;
          if (prolong) for (int q = 0; q < nfq; ++q) var_face[q] = coarse[v*nfq + q];
          for (int d = 0; d < ND - 1; ++d) {
            if (str[d]) {
              for (int q = 0; q < nfq; ++q) {
                if (prolong) var_face[q] *= 1 + scale;
                else var_face[q] /= 1 + scale;
              }
            } else {
              const int pw = ND - 2 - d;
              const int face_stride = str[ND - 2] ? 1 : ipow(2, pw);
              const int qstride = ipow(RS, pw);
              const int i_half = (i_face/face_stride)%2;
              const double* mat = (prolong ? t.prolong : t.restrict_) + i_half*RS*RS;
              for (int outer = 0; outer < nfq/(RS*qstride); ++outer) {
                for (int inner = 0; inner < qstride; ++inner) {
                  double row[RS], res[RS];
                  for (int k = 0; k < RS; ++k) row[k] = var_face[(outer*RS + k)*qstride + inner];
                  for (int i = 0; i < RS; ++i) {
                    double acc = 0.;
                    for (int j = 0; j < RS; ++j) acc += mat[i*RS + j]*row[j];
                    res[i] = acc;
                  }
                  for (int k = 0; k < RS; ++k) var_face[(outer*RS + k)*qstride + inner] = res[k];
                }
              }
            }
          }
          if (!prolong) for (int q = 0; q < nfq; ++q) coarse[v*nfq + q] += var_face[q];
        }
      }
    }
  }

  // ---------------------------------------------------------------- Max_dt
  // Spatial::Max_dt::operator() (include/Spatial.hpp:784-828)
  double max_dt(bool viscous, double msc, double msd, bool local_time,
                const hexed_transport& visc, const hexed_transport& cond) const
  {
    const double max_cfl_c = t.max_cfl*msc;
    const double max_cfl_d = -2/t.min_eig_diffusion*msd;
    double dt = std::numeric_limits<double>::max();
    #pragma omp parallel for reduction(min:dt)
    for (int e = 0; e < n_elem(); ++e) {
      double* state = elem(e);
      double* tss = state + nv*nq;
      const double* vt = m.vert_tss + (size_t)e*nvert;
      for (int q = 0; q < nq; ++q) {
        double vals[nvert];
        for (int i = 0; i < nvert; ++i) vals[i] = vt[i];
        int stride = nvert;
        for (int d = 0; d < ND; ++d) {
          double coord = t.node[(q/ipow(RS, ND - 1 - d))%RS];
          stride /= 2;
          for (int i = 0; i < stride; ++i) vals[i] += coord*(vals[i + stride] - vals[i]);
        }
        double spacing = vals[0];    // math::interp (include/math.hpp:207-218)
        double s[nv + 2];
        for (int v = 0; v < nv; ++v) s[v] = state[v*nq + q];
        s[nv] = state[(nv + 1)*nq + q];
        s[nv + 1] = state[(nv + 2)*nq + q];
        double scale = 0;
        if (fta) {
          scale += 1./max_cfl_d/spacing/spacing;   // Fix_therm_admis: diffusivity 1, no convection
        } else {
          scale += char_speed(s)/max_cfl_c/spacing;
        }
        if (viscous && !fta) {
          Conv c = scalars_conv(s);
          Diff df = scalars_diff(s, c, visc, cond);
          double diffusivity = std::abs(df.laplacian_av) + std::max(std::abs(df.bulk_av) + df.mu/c.mass, df.energy_cond/c.mass);
          scale += diffusivity/max_cfl_d/spacing/spacing;
        }
        if (local_time) tss[q] = 1./scale;
        else {
          tss[q] = 1.;
          dt = std::min(dt, 1./scale);
        }
      }
    }
    return local_time ? 1. : dt;
  }

  // ---------------------------------------------------------------- boundary conditions
  // Navier_stokes::Pde::Characteristics (include/pde.hpp:182-256) plus apply_char
  // (src/Boundary_condition.cpp:82-95).
  struct Characteristics {
    double vals[3], vecs[3][3], dir[ND], mass, veloc[ND];
    double lu[3][3]; int piv[3];
    double nrml(const double* v) const { double r = 0.; for (int d = 0; d < ND; ++d) r += dir[d]*v[d]; return r; }
    void tang(const double* v, double* out) const { double n = nrml(v); for (int d = 0; d < ND; ++d) out[d] = v[d] - dir[d]*n; }
    Characteristics(const double* state, const double* direction)
    {
      double nsq = 0.;
      for (int d = 0; d < ND; ++d) nsq += direction[d]*direction[d];
      double norm = std::sqrt(nsq);
      for (int d = 0; d < ND; ++d) dir[d] = direction[d]/norm;
      mass = state[ND];
      for (int d = 0; d < ND; ++d) veloc[d] = state[d]/mass;
      double vsq = 0.;
      for (int d = 0; d < ND; ++d) vsq += veloc[d]*veloc[d];
      double pres = .4*(state[ND + 1] - .5*mass*vsq);
      double sound_speed = std::sqrt(1.4*std::max(pres, 0.)/mass);
      vals[2] = nrml(veloc);
      vals[0] = vals[2] - sound_speed;
      vals[1] = vals[2] + sound_speed;
      double d_mass = 1;
      for (int sign = 0; sign < 2; ++sign) {
        double d_veloc = (2*sign - 1)*sound_speed/mass*d_mass;
        double d_pres = 1.4*pres/mass*d_mass;
        vecs[0][sign] = d_mass*vals[2] + mass*d_veloc;
        vecs[1][sign] = d_mass;
        vecs[2][sign] = d_pres/.4 + .5*d_mass*vsq + mass*vals[2]*d_veloc;
      }
      vecs[0][2] = d_mass*vals[2];
      vecs[1][2] = d_mass;
      vecs[2][2] = .5*d_mass*vsq;
      // LU with partial pivoting of vecs
      for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) lu[i][j] = vecs[i][j];
      for (int i = 0; i < 3; ++i) piv[i] = i;
      for (int k = 0; k < 3; ++k) {
        int p = k;
        for (int i = k + 1; i < 3; ++i) if (std::abs(lu[i][k]) > std::abs(lu[p][k])) p = i;
        if (p != k) { for (int j = 0; j < 3; ++j) std::swap(lu[k][j], lu[p][j]); std::swap(piv[k], piv[p]); }
        for (int i = k + 1; i < 3; ++i) {
          double f = lu[k][k] != 0. ? lu[i][k]/lu[k][k] : 0.;
          lu[i][k] = f;
          for (int j = k + 1; j < 3; ++j) lu[i][j] -= f*lu[k][j];
        }
      }
    }
    void solve(const double* b, double* x) const
    {
      double y[3];
      for (int i = 0; i < 3; ++i) {
        double acc = b[piv[i]];
        for (int j = 0; j < i; ++j) acc -= lu[i][j]*y[j];
        y[i] = acc;
      }
      for (int i = 2; i >= 0; --i) {
        double acc = y[i];
        for (int j = i + 1; j < 3; ++j) acc -= lu[i][j]*x[j];
        x[i] = lu[i][i] != 0. ? acc/lu[i][i] : 0.;
      }
    }
    // decomp (pde.hpp:234-255): d[nv][3]
    void decomp(const double* state, double (*d)[3]) const
    {
      double mmtm[ND], tm[ND], tv[ND], corr[ND];
      for (int i = 0; i < ND; ++i) mmtm[i] = state[i];
      tang(mmtm, tm);
      tang(veloc, tv);
      for (int i = 0; i < ND; ++i) corr[i] = tm[i] - state[ND]*tv[i];
      double vc = 0.;
      for (int i = 0; i < ND; ++i) vc += veloc[i]*corr[i];
      double s1d[3] = {nrml(mmtm), state[ND], state[ND + 1] - vc};
      double eb[3];
      solve(s1d, eb);
      double ed[3][3];
      for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) ed[r][c] = vecs[r][c]*eb[c];
      for (int c = 0; c < 3; ++c) {
        d[ND][c] = ed[1][c];
        d[ND + 1][c] = ed[2][c];
        for (int i = 0; i < ND; ++i) d[i][c] = dir[i]*ed[0][c] + tv[i]*eb[c];
      }
      for (int i = 0; i < ND; ++i) d[i][2] += corr[i];
      d[ND + 1][2] += vc;
    }
  };

  static void apply_char(const double* state, const double* normal, int sign, const double* inside,
                         const double* outside, double* out)
  {
    Characteristics ch(state, normal);
    double di[nv][3], fo[nv][3];
    ch.decomp(inside, di);
    ch.decomp(outside, fo);
    for (int i = 0; i < 3; ++i) {
      if (sign*ch.vals[i] > 0) for (int r = 0; r < nv; ++r) di[r][i] = fo[r][i];
    }
    for (int r = 0; r < nv; ++r) {
      double acc = 0.;
      for (int c = 0; c < 3; ++c) acc += di[r][c];
      out[r] = acc;
    }
  }

  static void reflect_normal(double* gh, const double* nrml) // Boundary_condition.cpp:302-317
  {
    for (int q = 0; q < nfq; ++q) {
      double dot = 0., norm_sq = 0.;
      for (int d = 0; d < ND; ++d) {
        double n = nrml[d*nfq + q];
        dot += gh[d*nfq + q]*n;
        norm_sq += n*n;
      }
      for (int d = 0; d < ND; ++d) gh[d*nfq + q] -= 2*dot*nrml[d*nfq + q]/norm_sq;
    }
  }

  void copy_state(double* in, double* gh) const // Boundary_condition.cpp:12-22 (both slots)
  {
    std::memcpy(gh, in, sizeof(double)*2*nv*nfq);
  }

  // Thermal_bc (include/Boundary_condition.hpp:140-190; src/Boundary_condition.cpp:373-379)
  static double ghost_energy(const hexed_bc_spec& b, const double* s)
  {
    if (b.thermal_kind == HEXED_THERMAL_ENERGY) return b.thermal_value*s[nv - 2];
    return s[nv - 1];
  }
  static double ghost_heat_flux(const hexed_bc_spec& b, const double* s, double heat_flux)
  {
    if (b.thermal_kind == HEXED_THERMAL_ENERGY) return heat_flux;
    if (b.thermal_kind == HEXED_THERMAL_HEAT_FLUX) return b.thermal_value;
    double temp = s[nv - 1]*.4/s[nv - 2]/specific_gas_air;
    const double sb = 2*ipow_d(M_PI, 5)*ipow_d(1.380649e-23, 4)/(15*ipow_d(299792458., 2)*ipow_d(6.62607015e-34, 3));
    double radiative = b.emissivity*sb*ipow_d(temp, 4);
    double conductive = b.heat_transfer_coef*(temp - b.temperature);
    return radiative + conductive;
  }
  static double ipow_d(double x, int e) { double r = 1; for (int i = 0; i < e; ++i) r *= x; return r; }

  void apply_state_bc(int i) const
  {
    const int* c = m.bc_con + 4*i;
    const hexed_bc_spec& b = m.bc_spec[c[3]];
    int ifs = (c[2] >> 2) & 1;
    double* in = slot(c[0], false);
    double* gh = slot(c[1], false);
    if (fta) {   // Solver::fix_admissibility (src/Solver.cpp:1067-1072): ghost face = inside face
      for (int k = 0; k < nv*nfq; ++k) gh[k] = in[k];
      return;
    }
    const double* nrml = m.bc_nrml + (size_t)i*ND*nfq;
    double* sc = m.bc_cache + (size_t)i*2*nv*nfq;
    switch (b.kind) {
      case HEXED_BC_FREESTREAM:
        for (int v = 0; v < nv; ++v) for (int q = 0; q < nfq; ++q) gh[v*nfq + q] = b.freestream[v];
        break;
      case HEXED_BC_RIEMANN_INVARIANTS: {
        int sign = 1 - 2*ifs;
        for (int q = 0; q < nfq; ++q) {
          double inside[nv], n[ND], st[nv];
          for (int v = 0; v < nv; ++v) inside[v] = in[v*nfq + q];
          for (int d = 0; d < ND; ++d) n[d] = nrml[d*nfq + q];
          apply_char(inside, n, sign, inside, b.freestream, st);
          st[ND] = std::max(st[ND], inside[ND]/2);
          double sq = 0., isq = 0.;
          for (int d = 0; d < ND; ++d) { sq += st[d]*st[d]; isq += inside[d]*inside[d]; }
          double kin = .5*sq/st[ND];
          double ikin = .5*isq/inside[ND];
          st[ND + 1] = std::max(kin + std::max(st[ND + 1] - kin, (inside[ND + 1] - ikin)/2), 0.);
          for (int v = 0; v < nv; ++v) gh[v*nfq + q] = st[v];
        }
        for (int k = 0; k < nv*nfq; ++k) sc[k] = in[k];
        break;
      }
      case HEXED_BC_NONPENETRATION:
        for (int k = 0; k < nv*nfq; ++k) gh[k] = in[k];
        reflect_normal(gh, nrml);
        break;
      case HEXED_BC_COPY:
      case HEXED_BC_OUTFLOW:
        copy_state(in, gh);
        break;
      case HEXED_BC_PRESSURE_OUTFLOW: {
        int sign = 2*ifs - 1;
        for (int q = 0; q < nfq; ++q) {
          double inside[nv], n[ND];
          for (int v = 0; v < nv; ++v) inside[v] = in[v*nfq + q];
          for (int d = 0; d < ND; ++d) n[d] = nrml[d*nfq + q];
          double dot = 0., nsq = 0., msq = 0.;
          for (int d = 0; d < ND; ++d) { dot += inside[d]*n[d]; nsq += n[d]*n[d]; msq += inside[d]*inside[d]; }
          double nrml_veloc = dot/inside[ND]/std::sqrt(nsq);
          double kin = .5*msq/inside[ND];
          double pres = std::max(.4*(inside[ND + 1] - kin), 0.);
          double sound = std::sqrt(1.4*pres/inside[ND]);
          double ghost[nv];
          for (int v = 0; v < nv; ++v) ghost[v] = inside[v];
          if (nrml_veloc*sign < sound) ghost[ND + 1] = b.pressure/.4 + kin;
          for (int v = 0; v < nv; ++v) gh[v*nfq + q] = ghost[v];
        }
        break;
      }
      case HEXED_BC_NO_SLIP: {
        for (int k = 0; k < ND*nfq; ++k) gh[k] = -in[k];
        for (int k = ND*nfq; k < (ND + 1)*nfq; ++k) gh[k] = in[k];
        for (int q = 0; q < nfq; ++q) {
          double s[nv];
          for (int v = 0; v < nv; ++v) s[v] = in[v*nfq + q];
          double ge = ghost_energy(b, s);
          gh[(ND + 1)*nfq + q] = ge*ge/s[nv - 1];
        }
        for (int k = 0; k < nv*nfq; ++k) sc[k] = (gh[k] + in[k])/2;
        break;
      }
    }
  }

  void apply_state_bcs() const
  {
    #pragma omp parallel for
    for (int i = 0; i < m.n_bc_con; ++i) apply_state_bc(i);
  }

  void apply_flux_bc(int i) const // Solver::apply_flux_bcs (src/Solver.cpp:69-81)
  {
    const int* c = m.bc_con + 4*i;
    const hexed_bc_spec& b = m.bc_spec[c[3]];
    int ifs = (c[2] >> 2) & 1;
    double* in_l = slot(c[0], true);
    double* gh_l = slot(c[1], true);
    if (fta) {   // Solver::apply_fta_flux_bcs (src/Solver.cpp:103-114)
      for (int k = 0; k < nv*nfq; ++k) gh_l[k] = -in_l[k];
      return;
    }
    const double* nrml = m.bc_nrml + (size_t)i*ND*nfq;
    double* sc = m.bc_cache + (size_t)i*2*nv*nfq;
    double* fc = sc + nv*nfq;
    for (int k = 0; k < nv*nfq; ++k) fc[k] = in_l[k];
    switch (b.kind) {
      case HEXED_BC_FREESTREAM:
      case HEXED_BC_COPY:
        copy_state(slot(c[0], false), slot(c[1], false));
        break;
      case HEXED_BC_RIEMANN_INVARIANTS: {
        int sign = 1 - 2*ifs;
        double zero[nv] = {};
        for (int q = 0; q < nfq; ++q) {
          double inside[nv], cache[nv], n[ND], st[nv];
          for (int v = 0; v < nv; ++v) { inside[v] = in_l[v*nfq + q]; cache[v] = sc[v*nfq + q]; }
          for (int d = 0; d < ND; ++d) n[d] = nrml[d*nfq + q];
          apply_char(cache, n, sign, zero, inside, st);
          for (int v = 0; v < nv; ++v) gh_l[v*nfq + q] = st[v];
        }
        break;
      }
      case HEXED_BC_NONPENETRATION:
        for (int k = 0; k < nv*nfq; ++k) gh_l[k] = -in_l[k];
        reflect_normal(gh_l, nrml);
        break;
      case HEXED_BC_OUTFLOW:
      case HEXED_BC_PRESSURE_OUTFLOW:
        for (int k = 0; k < nv*nfq; ++k) gh_l[k] = -in_l[k];
        break;
      case HEXED_BC_NO_SLIP: {
        for (int k = 0; k < ND*nfq; ++k) gh_l[k] = in_l[k];
        for (int k = ND*nfq; k < (ND + 1)*nfq; ++k) gh_l[k] = -in_l[k];
        for (int q = 0; q < nfq; ++q) {
          int k = q + (ND + 1)*nfq;
          double normal = 0;
          for (int d = 0; d < ND; ++d) { double n = nrml[d*nfq + q]; normal += n*n; }
          normal = std::sqrt(normal);
          int flux_sign = 2*ifs - 1;
          double s[nv];
          for (int v = 0; v < nv; ++v) s[v] = sc[v*nfq + q];
          gh_l[k] = b.coercion*(normal*flux_sign*ghost_heat_flux(b, s, in_l[k]*flux_sign/normal) - in_l[k]) + in_l[k];
        }
        break;
      }
    }
  }

  void apply_flux_bcs() const
  {
    #pragma omp parallel for
    for (int i = 0; i < m.n_bc_con; ++i) apply_flux_bc(i);
  }

  // ---------------------------------------------------------------- kernel sequences
  // compute_euler (src/kernels_convective.cpp:8-19)
  void compute_euler(double dt, int stage, bool cr, bool uf) const
  {
    hexed_transport inv{0., 0., 1., 1., 0};
    neighbor(false);
    refine(false, true, false);
    local(false, dt, stage, cr, uf, inv, inv);
    refine(true, false, false);
  }
  // compute_navier_stokes (src/kernels_diffusive.cpp:8-32)
  void compute_navier_stokes(double dt, int stage, bool cr, bool uf,
                             const hexed_transport& visc, const hexed_transport& cond) const
  {
    neighbor(true);
    refine(false, true, false);
    refine(false, false, true);
    local(true, dt, stage, cr, uf, visc, cond);
    if (!stage) {
      refine(true, true, true);
      apply_flux_bcs();
      neighbor_reconcile();
      refine(false, true, true);
      reconcile_ldg_flux(dt, cr, uf);
    }
    refine(true, false, false);
  }

  // Stab_art_visc (src/stabilizing_art_visc.cpp:26-60) for one element: the uncertainty
  double stab_uncert(int e, double char_speed) const
  {
    const double* state = elem(e);
    double qw[nq], fw[nfq], proj[RS];
    for (int q = 0; q < nq; ++q) {
      double p = 1.;
      for (int d = 0; d < ND; ++d) p *= t.weight[(q/ipow(RS, ND - 1 - d))%RS];
      qw[q] = p;
    }
    for (int r = 0; r < nfq; ++r) {
      double p = 1.;
      for (int d = 0; d < ND - 1; ++d) p *= t.weight[(r/ipow(RS, ND - 2 - d))%RS];
      fw[r] = p;
    }
    for (int i = 0; i < RS; ++i) proj[i] = t.ortho[(RS - 1)*RS + i]*t.weight[i];
    double iv[nq];
    double norm_sq = 0;
    for (int q = 0; q < nq; ++q) {
      iv[q] = 1./state[ND*nq + q];
      norm_sq += iv[q]*iv[q]*qw[q];
    }
    double nonsmooth = 0;
    for (int d = 0; d < ND; ++d) {
      for (int r = 0; r < nfq; ++r) {
        double dot = 0.;
        for (int i = 0; i < RS; ++i) dot += iv[row_qpoint(d, r, i)]*proj[i];
        nonsmooth += dot*dot*fw[r];
      }
    }
    nonsmooth /= norm_sq*ND;
    const double ramp_center = -4.25*std::log(RS - 1)/std::log(10);
    const double half_width = 0.5;
    double indicator = std::log(nonsmooth)/std::log(10);
    if (indicator <= ramp_center - half_width) indicator = 0;
    else if (indicator < ramp_center + half_width)
      indicator = .5*(1 + std::sin(M_PI*(indicator - ramp_center)/2/half_width));
    else indicator = 1;
    return (RS - 1)*char_speed*m.nom_size[e]*indicator;
  }

  // Solver::set_art_visc_admis (src/Solver.cpp:636-658): uncertainty, vertex maximum
  // (share_vertex_data with Vertex::vector_max), multilinear interpolation of the vertex
  // values to the qpoints (Gauss_lobatto(2).interpolate + hypercube_matvec) into the
  // Laplacian AV row.
  void set_art_visc_admis(double char_speed) const
  {
    std::vector<double> unc(n_elem());
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) unc[e] = stab_uncert(e, char_speed);
    std::vector<double> vmax(m.n_vert, -std::numeric_limits<double>::infinity());
    for (int e = 0; e < n_elem(); ++e)
      for (int v = 0; v < nvert; ++v) {
        double& x = vmax[m.vert_id[e*nvert + v]];
        x = std::max(x, unc[e]);
      }
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) {
      double* lap = elem(e) + (nv + 2)*nq;
      for (int q = 0; q < nq; ++q) {
        double vals[nvert];
        for (int v = 0; v < nvert; ++v) vals[v] = vmax[m.vert_id[e*nvert + v]];
        // contract the last reference dimension first, as hypercube_matvec does
        int n = nvert;
        for (int d = ND - 1; d >= 0; --d) {
          const double x = t.node[(q/ipow(RS, ND - 1 - d))%RS];
          for (int i = 0; i < n/2; ++i) vals[i] = (1. - x)*vals[2*i] + x*vals[2*i + 1];
          n /= 2;
        }
        lap[q] = vals[0];
      }
    }
  }

  // ---------------------------------------------------------------- admissibility
  // Solver::is_admissible (src/Solver.cpp:921-959) with thermo::admissible (src/thermo.cpp:6-18):
  // density and energy positive at every point of every element state, element face and
  // fine mortar face; record[e] = 1 marks an inadmissible element. *finite = false if any value
  // is not finite (the reference asserts there).
  bool is_admissible(std::vector<int>& record, bool* finite) const
  {
    record.assign(n_elem(), 0);
    bool admiss = true, fin = true;
    auto check = [&](const double* data, int n_point, int stride) {
      bool a = true;
      for (int q = 0; q < n_point; ++q) {
        a = a && (data[ND*stride + q] > 0.) && (data[(ND + 1)*stride + q] > 0.);
        for (int v = 0; v < nv; ++v) fin = fin && std::isfinite(data[v*stride + q]);
      }
      return a;
    };
    for (int e = 0; e < n_elem(); ++e) {
      bool ea = check(elem(e), nq, nq);
      for (int i = 0; i < 2*ND; ++i) ea = check(face(e, i, false), nfq, nfq) && ea;
      if (!ea) record[e] = 1;
      admiss = admiss && ea;
    }
    for (int i = 0; i < m.n_ref_face; ++i) {
      const int* rf = m.ref_face + 7*i;
      int n_fine = nvert/2;
      for (int d = 0; d < ND - 1; ++d) n_fine /= 1 + (rf[5 + d] != 0);
      for (int k = 0; k < n_fine; ++k) admiss = check(slot(rf[1 + k], false), nfq, nfq) && admiss;
    }
    *finite = fin;
    return admiss;
  }

  // std::swap of the bulk and Laplacian artificial-viscosity rows (src/Solver.cpp:1033-1039)
  void swap_av() const
  {
    for (int e = 0; e < n_elem(); ++e) {
      double* st = elem(e);
      for (int q = 0; q < nq; ++q) std::swap(st[(nv + 1)*nq + q], st[(nv + 2)*nq + q]);
    }
  }

  // Solver::fix_admissibility's coefficient (src/Solver.cpp:990-1032): each element's record on
  // its vertices, vertex maximum, the maximum over each element's vertices, vertex maximum
  // again, multilinear interpolation into the Laplacian AV row (skipped without a vertex table)
  void fix_admis_coef(const std::vector<int>& record) const
  {
    if (m.n_vert <= 0 || !m.vert_id) return;
    std::vector<double> vmax(m.n_vert, 0.), emax(n_elem());
    for (int e = 0; e < n_elem(); ++e)
      for (int v = 0; v < nvert; ++v) { double& x = vmax[m.vert_id[e*nvert + v]]; x = std::max(x, double(record[e])); }
    for (int e = 0; e < n_elem(); ++e) {
      double mx = 0.;
      for (int v = 0; v < nvert; ++v) mx = std::max(mx, vmax[m.vert_id[e*nvert + v]]);
      emax[e] = mx;
    }
    std::fill(vmax.begin(), vmax.end(), 0.);
    for (int e = 0; e < n_elem(); ++e)
      for (int v = 0; v < nvert; ++v) { double& x = vmax[m.vert_id[e*nvert + v]]; x = std::max(x, emax[e]); }
    for (int e = 0; e < n_elem(); ++e) {
      double* lap = elem(e) + (nv + 2)*nq;
      for (int q = 0; q < nq; ++q) {
        double vals[nvert];
        for (int v = 0; v < nvert; ++v) vals[v] = vmax[m.vert_id[e*nvert + v]];
        int n = nvert;
        for (int d = ND - 1; d >= 0; --d) {
          const double x = t.node[(q/ipow(RS, ND - 1 - d))%RS];
          for (int i = 0; i < n/2; ++i) vals[i] = (1. - x)*vals[2*i] + x*vals[2*i + 1];
          n /= 2;
        }
        lap[q] = vals[0];
      }
    }
  }

  // Solver::fix_admissibility (src/Solver.cpp:961-1095); returns the iteration count the
  // reference returns, or -1 for a non-finite state and -2 past 100000 iterations (where the
  // reference asserts). The flow's Max_dt closing each iteration uses the update parameters p.
  int fix_admissibility(const hexed_update_params& p, double stability_ratio, double (*cheby)(int, int)) const
  {
    const hexed_transport inv{0., 0., 1., 1., 0};
    std::vector<int> record;
    int iter;
    int n_iters = std::numeric_limits<int>::max();
    for (iter = 0; iter < n_iters; ++iter) {
      if (iter >= 100000) return -2;
      bool finite;
      const bool adm = is_admissible(record, &finite);
      if (!finite) return -1;
      if (adm) {
        if (iter) n_iters = std::min(n_iters, 2*iter);
        else {
          ++iter;
          break;
        }
      } else {
        n_iters = std::numeric_limits<int>::max();
      }
      fix_admis_coef(record);
      swap_av();
      fta = true;
      max_dt(true, stability_ratio, stability_ratio, true, inv, inv);
      const double linear = 1., quadratic = 1./8/0.9;
      double step[2];
      step[1] = (linear + std::sqrt(linear*linear - 4*quadratic))/2.;
      step[0] = quadratic/step[1];
      for (double st : step) {
        apply_state_bcs();
        compute_navier_stokes(st, 0, false, false, inv, inv);
      }
      fta = false;
      const double max_cheby = cheby(p.n_cheby_flow, p.n_cheby_flow - 1);
      max_dt(p.use_ldg, p.max_safety/max_cheby, p.max_safety, p.local_time, p.visc, p.cond);
      swap_av();
    }
    --iter;
    return iter;
  }

  // integral_field of Physical_residual^2 (src/Solver.cpp:1113-1131, src/Qpoint_func.cpp:37-45)
  void residual_norm(double* out) const
  {
    double w[nq];
    for (int q = 0; q < nq; ++q) {
      double p = 1.;
      for (int d = 0; d < ND; ++d) p *= t.weight[(q/ipow(RS, ND - 1 - d))%RS];
      w[q] = p;
    }
    double acc[nv] = {};
    for (int e = 0; e < n_elem(); ++e) {
      double vol = 1.;
      for (int d = 0; d < ND; ++d) vol *= m.nom_size[e];
      const double* st = elem(e);
      const double* rc = rcache(e);
      const double* det = e >= m.n_car_elem ? m.jac + (size_t)(e - m.n_car_elem)*(ND*ND + 1)*nq + ND*ND*nq : nullptr;
      for (int q = 0; q < nq; ++q) {
        double tss = st[nv*nq + q];
        double jd = det ? det[q] : 1.;
        for (int v = 0; v < nv; ++v) {
          double r = rc[v*nq + q]/tss;
          acc[v] += w[q]*vol*(r*r)*jd;
        }
      }
    }
    double mom = 0.;
    for (int d = 0; d < ND; ++d) mom += acc[d];
    out[0] = std::sqrt(mom);
    out[1] = std::sqrt(acc[ND]);
    out[2] = std::sqrt(acc[ND + 1]);
  }
};

template <int ND, int RS>
struct Dispatch;

template <typename F>
int dispatch(const hexed_mesh_desc* m, F&& f)
{
  if (!m) return HEXED_ERR_INVALID;
  switch (m->n_dim*16 + m->row_size) {
#define HEXED_D(nd, rs) case nd*16 + rs: { K<nd, rs> k(*m); f(k); return HEXED_OK; }
    HEXED_D(2, 2) HEXED_D(2, 3) HEXED_D(2, 4) HEXED_D(2, 5) HEXED_D(2, 6) HEXED_D(2, 7) HEXED_D(2, 8)
    HEXED_D(3, 2) HEXED_D(3, 3) HEXED_D(3, 4) HEXED_D(3, 5) HEXED_D(3, 6) HEXED_D(3, 7) HEXED_D(3, 8)
#undef HEXED_D
  }
  return HEXED_ERR_INVALID;
}

// chebyshev_step (src/math.cpp:104-107)
double chebyshev_step(int n_steps, int i_step)
{
  return 1/(1 - std::cos((n_steps - i_step - 0.5)*M_PI/n_steps));
}

// ---------------------------------------------------------------- smoothness-based AV
// Solver::update_art_visc_smoothness (src/Solver.cpp:457-582): the Spatial kernels applied to
// pde::Advection and pde::Smooth_art_visc (include/pde.hpp:265-431), hanging faces included.
// Storage beside the arena:
//  * aux  [n_elem][4 + 2*row_size][nq]: the art_visc_forcing rows (Storage_params::n_forcing
//    = 4), the advection state (row_size rows) and its residual cache (row_size rows: the
//    element's residual_cache, which the reference sizes for max(n_var, row_size) rows);
//  * face [n_slot][max(2*nv, nd + row_size)*nfq]: one face slot per arena slot, the size of a
//    Face_connection face (include/connection.hpp:58-66); the LDG half starts at nv*nfq as
//    in Element::face (src/Element.cpp:189). The reference keeps these traces in the flow's
//    face storage; the flow's update rewrites every trace it reads before reading it.
// The flow state is used in place: the momentum rows are divided by sqrt(2 rho E) for the
// advection velocity and multiplied back at the end (the reference does the same, so the
// momentum keeps the same last bits); the time-step-scale row is overwritten by the
// pseudo-time steps; the bulk AV row receives the coefficient.
template <int ND, int RS>
struct Sav
{
  using KK = K<ND, RS>;
  static constexpr int nq = KK::nq, nfq = KK::nfq, nv = KK::nv, nvert = KK::nvert;
  static constexpr int n_forcing = 4;
  static constexpr int n_adv = RS;                       // Storage_params::n_advection
  static constexpr int n_aux = n_forcing + 2*n_adv;
  static constexpr int n_adv_extrap = ND + n_adv;        // pde::Advection::n_extrap
  static constexpr int n_sav = 3;                        // pde::Smooth_art_visc::n_extrap, n_update
  static constexpr int slot_dof = (2*nv > n_adv_extrap ? 2*nv : n_adv_extrap)*nfq;

  const KK& k;
  const hexed_mesh_desc& m;
  double* aux;
  double* sf;
  const oracle_sav_params& p;
  double adv_node[RS];   // pde::Advection::_nodes = 2*(Gauss-Legendre nodes) - 1 (pde.hpp:281)

  Sav(const KK& kk, double* aux_, double* face_, const oracle_sav_params& par)
  : k{kk}, m{kk.m}, aux{aux_}, sf{face_}, p{par}
  {
    for (int i = 0; i < RS; ++i) adv_node[i] = 2*k.t.node[i] - 1.;
  }

  double* forcing(int e) const { return aux + (size_t)e*n_aux*nq; }
  double* adv(int e) const { return forcing(e) + n_forcing*nq; }
  double* adv_cache(int e) const { return adv(e) + n_adv*nq; }
  double* slot(int s, bool ldg) const { return sf + (size_t)s*slot_dof + ldg*nv*nfq; }
  double* face(int e, int i, bool ldg) const { return slot(e*2*ND + i, ldg); }
  int n_elem() const { return k.n_elem(); }
  // Prolong_refined / Restrict_refined of the Pde's n_extrap face variables on these slots
  void refine(int n_var, bool prolong, bool scale, bool offset) const
  {
    k.refine_slots(sf, slot_dof, n_var, prolong, scale, offset);
  }
  const double* jac(int e) const { return m.jac + (size_t)(e - m.n_car_elem)*(ND*ND + 1)*nq; }

  // mesh spacing at a qpoint: math::interp of the vertex time-step scales (include/math.hpp:207-218)
  double spacing(int e, int q) const
  {
    const double* vt = m.vert_tss + (size_t)e*nvert;
    double vals[nvert];
    for (int i = 0; i < nvert; ++i) vals[i] = vt[i];
    int stride = nvert;
    for (int d = 0; d < ND; ++d) {
      double coord = k.t.node[(q/ipow(RS, ND - 1 - d))%RS];
      stride /= 2;
      for (int i = 0; i < stride; ++i) vals[i] += coord*(vals[i + stride] - vals[i]);
    }
    return vals[0];
  }

  // Spatial<pde::Advection>::Max_dt with local time stepping (include/Spatial.hpp:784-828):
  // char_speed = max(1, |velocity|) (pde.hpp:343-346), no diffusion
  void max_dt_advection() const
  {
    const double max_cfl_c = k.t.max_cfl*p.advect_safety;
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) {
      double* state = k.elem(e);
      for (int q = 0; q < nq; ++q) {
        double sq = 0.;
        for (int d = 0; d < ND; ++d) sq += state[d*nq + q]*state[d*nq + q];
        double cs = std::max(1., std::sqrt(sq));
        double scale = 0;
        scale += cs/max_cfl_c/spacing(e, q);
        state[nv*nq + q] = 1./scale;
      }
    }
  }

  // Spatial<pde::Smooth_art_visc>::Max_dt with local time stepping: diffusivity 1, no convection
  void max_dt_smooth_av() const
  {
    const double max_cfl_d = -2/k.t.min_eig_diffusion*p.diff_safety;
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) {
      double* state = k.elem(e);
      for (int q = 0; q < nq; ++q) {
        double sp = spacing(e, q);
        double scale = 0;
        scale += 1./max_cfl_d/sp/sp;
        state[nv*nq + q] = 1./scale;
      }
    }
  }

  // Spatial::Write_face (include/Spatial.hpp:41-57) of n_var rows of `rows` into the element's faces
  void write_face_rows(int e, const double* const* rows, int n_var) const
  {
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        for (int v = 0; v < n_var; ++v) {
          for (int s = 0; s < 2; ++s) {
            double acc = 0.;
            for (int i = 0; i < RS; ++i) acc += k.t.bound[s*RS + i]*rows[v][KK::row_qpoint(d, i_fq, i)];
            face(e, 2*d + s, false)[v*nfq + i_fq] = acc;
          }
        }
      }
    }
  }
  // pde::Advection::fetch_extrap (pde.hpp:284-290): the velocity rows, then the advection state
  void write_face_advection(int e) const
  {
    const double* rows[n_adv_extrap];
    for (int d = 0; d < ND; ++d) rows[d] = k.elem(e) + d*nq;
    for (int a = 0; a < n_adv; ++a) rows[ND + a] = adv(e) + a*nq;
    write_face_rows(e, rows, n_adv_extrap);
  }
  // pde::Smooth_art_visc::fetch_extrap (pde.hpp:372-377): forcing rows 1-3
  void write_face_smooth_av(int e) const
  {
    const double* rows[n_sav];
    for (int v = 0; v < n_sav; ++v) rows[v] = forcing(e) + (1 + v)*nq;
    write_face_rows(e, rows, n_sav);
  }

  // Flow_bc::apply_advection and its overrides (src/Boundary_condition.cpp:24-41, 346-368,
  // 429-448, 460-463)
  void apply_advection_bc(int i) const
  {
    const int* c = m.bc_con + 4*i;
    const hexed_bc_spec& b = m.bc_spec[c[3]];
    double* in = slot(c[0], false);
    double* gh = slot(c[1], false);
    switch (b.kind) {
      case HEXED_BC_NONPENETRATION: {
        const double* nrml = m.bc_nrml + (size_t)i*ND*nfq;
        for (int q = 0; q < nfq; ++q) {
          double dot = 0., nsq = 0.;
          for (int d = 0; d < ND; ++d) {
            double n = nrml[d*nfq + q];
            dot += in[d*nfq + q]*n;
            nsq += n*n;
          }
          for (int d = 0; d < ND; ++d) gh[d*nfq + q] = in[d*nfq + q] - 2*dot*nrml[d*nfq + q]/nsq;
          for (int a = 0; a < n_adv; ++a) gh[(ND + a)*nfq + q] = in[(ND + a)*nfq + q];
        }
        break;
      }
      case HEXED_BC_NO_SLIP:
        for (int k2 = 0; k2 < ND*nfq; ++k2) gh[k2] = -in[k2];
        for (int k2 = ND*nfq; k2 < n_adv_extrap*nfq; ++k2) gh[k2] = in[k2];
        break;
      case HEXED_BC_COPY:
        // copy_state (src/Boundary_condition.cpp:12-22): both halves of the face, n_var*nfq each
        for (int k2 = 0; k2 < 2*nv*nfq; ++k2) gh[k2] = in[k2];
        break;
      default:
        // velocity as inside; advected scalars mirrored about 1
        for (int k2 = 0; k2 < ND*nfq; ++k2) gh[k2] = in[k2];
        for (int k2 = 0; k2 < n_adv*nfq; ++k2) gh[ND*nfq + k2] = 2. - in[ND*nfq + k2];
    }
  }

  // the three connection lists with the direction encoding of K::neighbor
  template <typename F>
  void for_connections(F&& f) const
  {
    #pragma omp parallel for
    for (int i = 0; i < m.n_car_con; ++i) {
      const int* c = m.car_con + 3*i;
      f(c[0], c[1], c[2] | (c[2] << 2) | (1 << 4), (const double*)nullptr);
    }
    #pragma omp parallel for
    for (int i = 0; i < m.n_def_con; ++i) {
      const int* c = m.def_con + 3*i;
      f(c[0], c[1], c[2], (const double*)(m.def_con_nrml + (size_t)i*ND*nfq));
    }
    #pragma omp parallel for
    for (int i = 0; i < m.n_bc_con; ++i) {
      const int* c = m.bc_con + 4*i;
      int d = c[2] & 3, ifs = (c[2] >> 2) & 1;
      f(c[0], c[1], d | (d << 2) | (ifs << 4) | ((!ifs) << 5), (const double*)(m.bc_nrml + (size_t)i*ND*nfq));
    }
  }

  static void signs(int dir, bool deformed, int* sign)
  {
    sign[0] = sign[1] = 1;
    if (deformed) {
      bool s0 = (dir >> 4) & 1, s1 = (dir >> 5) & 1;
      sign[0] = 1 - 2*(s0 == 0);
      sign[1] = 1 - 2*(s1 == 1);
    }
  }

  // Spatial<pde::Advection>::Neighbor (include/Spatial.hpp:613-705): local Lax-Friedrichs flux
  // of the advected scalars, written over the first row_size face variables of both sides
  void neighbor_advection_con(int slot0, int slot1, int dir, const double* nrml) const
  {
    const bool deformed = nrml != nullptr;
    int sign[2];
    signs(dir, deformed, sign);
    double* f0 = slot(slot0, false);
    double* f1 = slot(slot1, false);
    double out0[n_adv*nfq], out1[n_adv*nfq];
    for (int q = 0; q < nfq; ++q) {
      const int q1 = deformed ? KK::perm_index(dir, q) : q;
      double n[ND];
      if (deformed) for (int d = 0; d < ND; ++d) n[d] = sign[0]*nrml[d*nfq + q];
      else for (int d = 0; d < ND; ++d) n[d] = (d == (dir & 3)) ? 1. : 0.;
      double u[2][n_adv_extrap], fl[2][n_adv], cs[2];
      for (int v = 0; v < n_adv_extrap; ++v) { u[0][v] = f0[v*nfq + q]; u[1][v] = f1[v*nfq + q1]; }
      for (int side = 0; side < 2; ++side) {
        double nrml_veloc = 0, sq = 0.;
        for (int d = 0; d < ND; ++d) nrml_veloc += u[side][d]*n[d];
        for (int a = 0; a < n_adv; ++a) fl[side][a] = adv_node[a]*nrml_veloc*u[side][ND + a];
        for (int d = 0; d < ND; ++d) sq += u[side][d]*u[side][d];
        cs[side] = std::max(1., std::sqrt(sq));
      }
      double nn = 0.;
      for (int d = 0; d < ND; ++d) nn += n[d]*n[d];
      double mult = std::max(cs[0], cs[1])*std::sqrt(nn);
      for (int a = 0; a < n_adv; ++a) {
        double flux = .5*(fl[0][a] + fl[1][a] + mult*(u[0][ND + a] - u[1][ND + a]));
        out0[a*nfq + q] = sign[0]*flux;
        out1[a*nfq + q1] = sign[1]*flux;
      }
    }
    std::memcpy(f0, out0, sizeof(out0));
    std::memcpy(f1, out1, sizeof(out1));
  }

  // Spatial<pde::Advection>::Local (include/Spatial.hpp:326-509) for one element: convective
  // flux nodes_i*(v.n)*a_i, the source 2/advect_length in the first stage, and
  // Advection::write_update (pde.hpp:292-300): pseudo = 1 + 2*tss/advect_length, the first
  // stage sets a = (a + update)/pseudo, the second adds update/pseudo.
  void local_advection_elem(int e, bool deformed, int stage) const
  {
    double* state = k.elem(e);
    double* tss = state + nv*nq;
    double* a_st = adv(e);
    double* ref_state = adv_cache(e);
    const double d_pos = m.nom_size[e];
    const double* nrml = deformed ? jac(e) : nullptr;
    const double* det = deformed ? jac(e) + ND*ND*nq : nullptr;
    static thread_local std::vector<double> buf;
    buf.assign((size_t)(2*n_adv*nq + ND*n_adv*nq), 0.);
    double (*time_rate)[n_adv][nq] = reinterpret_cast<double (*)[n_adv][nq]>(buf.data());
    double (*flux)[n_adv][nq] = reinterpret_cast<double (*)[n_adv][nq]>(buf.data() + 2*n_adv*nq);
    for (int q = 0; q < nq; ++q) {
      for (int i = 0; i < ND; ++i) {
        double nrml_veloc = 0;
        for (int j = 0; j < ND; ++j)
          nrml_veloc += state[j*nq + q]*(deformed ? nrml[(i*ND + j)*nq + q] : (i == j ? 1. : 0.));
        for (int a = 0; a < n_adv; ++a) flux[i][a][q] = adv_node[a]*nrml_veloc*a_st[a*nq + q];
      }
      if (!stage) {
        double mult = d_pos;
        if (deformed) mult *= det[q];
        for (int a = 0; a < n_adv; ++a) time_rate[1][a][q] = mult*(2/p.advect_length);
      }
    }
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        for (int a = 0; a < n_adv; ++a) {
          double row_f[RS], face_f[2], der[RS];
          for (int i = 0; i < RS; ++i) row_f[i] = flux[d][a][KK::row_qpoint(d, i_fq, i)];
          for (int s = 0; s < 2; ++s) face_f[s] = face(e, 2*d + s, false)[a*nfq + i_fq];
          k.derivative(row_f, face_f, der);
          for (int i = 0; i < RS; ++i) {
            double& x = time_rate[0][a][KK::row_qpoint(d, i_fq, i)];
            x = 1.*x + -der[i];
          }
        }
      }
    }
    const double update_coef = stage ? 1.*k.t.step_ratio : 1.;
    for (int q = 0; q < nq; ++q) {
      double mult = update_coef*tss[q]/d_pos;
      if (deformed) mult /= det[q];
      const double pseudo = 1 + tss[q]*2/p.advect_length;
      for (int a = 0; a < n_adv; ++a) {
        double u = time_rate[0][a][q];
        if (stage) u -= ref_state[a*nq + q];
        else {
          ref_state[a*nq + q] = u;
          u += time_rate[1][a][q];
        }
        u *= mult;
        double& x = a_st[a*nq + q];
        if (!stage) x = (x + u)/pseudo;
        else x += u/pseudo;
      }
    }
    write_face_advection(e);
  }

  // compute_advection (src/kernels_convective.cpp:8-19), dt = 1
  void compute_advection(int stage) const
  {
    for_connections([&](int s0, int s1, int dir, const double* nrml) { neighbor_advection_con(s0, s1, dir, nrml); });
    refine(n_adv_extrap, false, true, false);
    #pragma omp parallel for
    for (int e = 0; e < m.n_car_elem; ++e) local_advection_elem(e, false, stage);
    #pragma omp parallel for
    for (int e = m.n_car_elem; e < n_elem(); ++e) local_advection_elem(e, true, stage);
    refine(n_adv_extrap, true, false, false);
  }

  // Spatial<pde::Smooth_art_visc>::Neighbor: the LDG average of the three traces on both sides
  void neighbor_smooth_av_con(int slot0, int slot1, int dir, const double* nrml) const
  {
    const bool deformed = nrml != nullptr;
    const double* f0 = slot(slot0, false);
    const double* f1 = slot(slot1, false);
    double* l0 = slot(slot0, true);
    double* l1 = slot(slot1, true);
    for (int q = 0; q < nfq; ++q) {
      const int q1 = deformed ? KK::perm_index(dir, q) : q;
      for (int v = 0; v < n_sav; ++v) {
        double avg = .5*(f0[v*nfq + q] + f1[v*nfq + q1]);
        l0[v*nfq + q] = avg;
        l1[v*nfq + q1] = avg;
      }
    }
  }

  // Spatial<pde::Smooth_art_visc>::Local (include/Spatial.hpp:326-509), first stage, for one
  // element. The unknowns are forcing rows 1-3; their flux is -gradient.normal, diffusivity 1;
  // the source of unknown i is f(forcing row i)/diff_time with f = |x| for rows 0 and 2 and
  // sqrt|x| for row 1 (pde.hpp:422-429); write_update adds (pde.hpp:379-387, not critical).
  void local_smooth_av_elem(int e, bool deformed, double dt, double diff_time) const
  {
    double* state = k.elem(e);
    double* tss = state + nv*nq;
    double* fc = forcing(e);
    const double d_pos = m.nom_size[e];
    const double* nrml = deformed ? jac(e) : nullptr;
    const double* det = deformed ? jac(e) + ND*ND*nq : nullptr;
    const double* face_nrml[6] = {};
    if (deformed) {
      const int ed = e - m.n_car_elem;
      for (int i = 0; i < 2*ND; ++i) face_nrml[i] = m.face_nrml + ((size_t)ed*2*ND + i)*ND*nfq;
    }
    double time_rate[2][n_sav][nq];
    double visc_storage[ND][n_sav][nq];
    for (int v = 0; v < n_sav; ++v) for (int q = 0; q < nq; ++q) {
      time_rate[0][v][q] = time_rate[1][v][q] = 0.;
      for (int d = 0; d < ND; ++d) visc_storage[d][v][q] = 0.;
    }
    // gradient times the Jacobian determinant (Spatial.hpp:371-402)
    for (int v = 0; v < n_sav; ++v) for (int q = 0; q < nq; ++q) time_rate[0][v][q] = fc[(1 + v)*nq + q];
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        double row_r[n_sav][RS], fs[n_sav][2];
        for (int v = 0; v < n_sav; ++v) {
          for (int i = 0; i < RS; ++i) row_r[v][i] = time_rate[0][v][KK::row_qpoint(d, i_fq, i)];
          for (int s = 0; s < 2; ++s) fs[v][s] = face(e, 2*d + s, true)[v*nfq + i_fq];
        }
        if (deformed) {
          for (int j = 0; j < ND; ++j) {
            double row_n[RS], face_n[2];
            for (int i = 0; i < RS; ++i) row_n[i] = nrml[(d*ND + j)*nq + KK::row_qpoint(d, i_fq, i)];
            for (int s = 0; s < 2; ++s) face_n[s] = face_nrml[2*d + s][j*nfq + i_fq];
            for (int v = 0; v < n_sav; ++v) {
              double row[RS], bound[2], der[RS];
              for (int i = 0; i < RS; ++i) row[i] = row_n[i]*row_r[v][i];
              for (int s = 0; s < 2; ++s) bound[s] = face_n[s]*fs[v][s];
              k.derivative(row, bound, der);
              for (int i = 0; i < RS; ++i) {
                double& x = visc_storage[j][v][KK::row_qpoint(d, i_fq, i)];
                x = 1.*x + der[i]/d_pos;
              }
            }
          }
        } else {
          for (int v = 0; v < n_sav; ++v) {
            double der[RS];
            k.derivative(row_r[v], fs[v], der);
            for (int i = 0; i < RS; ++i) {
              double& x = visc_storage[d][v][KK::row_qpoint(d, i_fq, i)];
              x = 0*x + der[i]/d_pos;
            }
          }
        }
      }
    }
    for (int v = 0; v < n_sav; ++v) for (int q = 0; q < nq; ++q) { time_rate[0][v][q] = 0; time_rate[1][v][q] = 0; }
    // flux and source (Spatial.hpp:405-442)
    for (int q = 0; q < nq; ++q) {
      double g[n_sav][ND];
      for (int d = 0; d < ND; ++d) for (int v = 0; v < n_sav; ++v) g[v][d] = visc_storage[d][v][q];
      if (deformed) for (int v = 0; v < n_sav; ++v) for (int d = 0; d < ND; ++d) g[v][d] /= det[q];
      for (int v = 0; v < n_sav; ++v) for (int i = 0; i < ND; ++i) {
        double acc = 0.;
        for (int j = 0; j < ND; ++j) acc += -g[v][j]*(deformed ? nrml[(i*ND + j)*nq + q] : (i == j ? 1. : 0.));
        visc_storage[i][v][q] = acc;
      }
      double mult = d_pos;
      if (deformed) mult *= det[q];
      for (int v = 0; v < n_sav; ++v) {
        double f = std::abs(fc[v*nq + q]);
        time_rate[1][v][q] = mult*(((v == 1) ? std::sqrt(f) : f)/diff_time);
      }
    }
    // residual (Spatial.hpp:445-470): interior divergence of the flux; the flux's face values
    // go to the LDG faces
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        for (int v = 0; v < n_sav; ++v) {
          double row_f[RS], der[RS];
          for (int i = 0; i < RS; ++i) row_f[i] = visc_storage[d][v][KK::row_qpoint(d, i_fq, i)];
          for (int s = 0; s < 2; ++s) {
            double acc = 0.;
            for (int i = 0; i < RS; ++i) acc += k.t.bound[s*RS + i]*row_f[i];
            face(e, 2*d + s, true)[v*nfq + i_fq] = acc;
          }
          k.derivative_interior(row_f, der);
          for (int i = 0; i < RS; ++i) {
            double& x = time_rate[1][v][KK::row_qpoint(d, i_fq, i)];
            x = 1.*x + -der[i];
          }
        }
      }
    }
    for (int q = 0; q < nq; ++q) {
      double mult = dt*tss[q]/d_pos;
      if (deformed) mult /= det[q];
      for (int v = 0; v < n_sav; ++v) {
        double u = time_rate[0][v][q];
        u += time_rate[1][v][q];
        u *= mult;
        fc[(1 + v)*nq + q] += u;
      }
    }
  }

  // Spatial::Neighbor_reconcile (include/Spatial.hpp:716-759) over the three LDG fluxes
  void neighbor_reconcile_smooth_av_con(int slot0, int slot1, int dir, const double* nrml) const
  {
    const bool deformed = nrml != nullptr;
    int sign[2];
    signs(dir, deformed, sign);
    double* l0 = slot(slot0, true);
    double* l1 = slot(slot1, true);
    double out0[n_sav*nfq], out1[n_sav*nfq];
    for (int q = 0; q < nfq; ++q) {
      const int q1 = deformed ? KK::perm_index(dir, q) : q;
      for (int v = 0; v < n_sav; ++v) {
        double a = l0[v*nfq + q], b = l1[v*nfq + q1];
        double avg = 0;
        avg += .5*sign[0]*a;
        avg += .5*sign[1]*b;
        out0[v*nfq + q] = sign[0]*avg - a;
        out1[v*nfq + q1] = sign[1]*avg - b;
      }
    }
    std::memcpy(l0, out0, sizeof(out0));
    std::memcpy(l1, out1, sizeof(out1));
  }

  // Spatial<pde::Smooth_art_visc>::Reconcile_ldg_flux (include/Spatial.hpp:543-594): lift of
  // the flux differences, then the critical write_update: add, then divide by
  // pseudo = 1 + tss*chebyshev_step/diff_time (pde.hpp:379-387); the traces are re-extrapolated
  void reconcile_smooth_av_elem(int e, bool deformed, double dt, double diff_time, double cheby) const
  {
    double* state = k.elem(e);
    double* tss = state + nv*nq;
    double* fc = forcing(e);
    const double d_pos = m.nom_size[e];
    const double* det = deformed ? jac(e) + ND*ND*nq : nullptr;
    double time_rate[n_sav][nq];
    for (int v = 0; v < n_sav; ++v) for (int q = 0; q < nq; ++q) time_rate[v][q] = 0.;
    for (int d = 0; d < ND; ++d) {
      for (int i_fq = 0; i_fq < nfq; ++i_fq) {
        for (int v = 0; v < n_sav; ++v) {
          double b0 = face(e, 2*d, true)[v*nfq + i_fq];
          double b1 = face(e, 2*d + 1, true)[v*nfq + i_fq];
          for (int i = 0; i < RS; ++i) {
            double l = 0.;
            l += k.lift[i][0]*b0;
            l += k.lift[i][1]*b1;
            double& x = time_rate[v][KK::row_qpoint(d, i_fq, i)];
            x = 1.*x + -l;
          }
        }
      }
    }
    for (int q = 0; q < nq; ++q) {
      double mult = dt*tss[q]/d_pos;
      if (deformed) mult /= det[q];
      const double pseudo = 1 + tss[q]*cheby/diff_time;
      for (int v = 0; v < n_sav; ++v) {
        double& x = fc[(1 + v)*nq + q];
        x += time_rate[v][q]*mult;
        x /= pseudo;
      }
    }
    write_face_smooth_av(e);
  }

  // compute_smooth_av (src/kernels_diffusive.cpp:8-30), first stage
  void compute_smooth_av(double dt, double diff_time, double cheby) const
  {
    for_connections([&](int s0, int s1, int dir, const double* nrml) { neighbor_smooth_av_con(s0, s1, dir, nrml); });
    refine(n_sav, false, true, false);
    refine(n_sav, false, false, true);
    #pragma omp parallel for
    for (int e = 0; e < m.n_car_elem; ++e) local_smooth_av_elem(e, false, dt, diff_time);
    #pragma omp parallel for
    for (int e = m.n_car_elem; e < n_elem(); ++e) local_smooth_av_elem(e, true, dt, diff_time);
    refine(n_sav, true, true, true);
    // Solver::apply_avc_diff_flux_bcs -> Flow_bc::flux_diffusion (src/Boundary_condition.cpp:54-60)
    #pragma omp parallel for
    for (int i = 0; i < m.n_bc_con; ++i) {
      const int* c = m.bc_con + 4*i;
      const double* in = slot(c[0], true);
      double* gh = slot(c[1], true);
      for (int k2 = 0; k2 < nv*nfq; ++k2) gh[k2] = -in[k2];
    }
    for_connections([&](int s0, int s1, int dir, const double* nrml) {
      neighbor_reconcile_smooth_av_con(s0, s1, dir, nrml);
    });
    refine(n_sav, false, true, true);
    #pragma omp parallel for
    for (int e = 0; e < m.n_car_elem; ++e) reconcile_smooth_av_elem(e, false, dt, diff_time, cheby);
    #pragma omp parallel for
    for (int e = m.n_car_elem; e < n_elem(); ++e) reconcile_smooth_av_elem(e, true, dt, diff_time, cheby);
    refine(n_sav, true, false, false);
  }

  // Solver::diffuse_art_visc (src/Solver.cpp:428-455)
  void diffuse_art_visc(double diff_time) const
  {
    max_dt_smooth_av();
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) write_face_smooth_av(e);
    refine(nv, true, false, false);   // compute_prolong: the flow's n_extrap = nv variables
    for (int i_iter = 0; i_iter < p.diff_iters; ++i_iter) {
      for (int i_cheby = 0; i_cheby < p.n_cheby; ++i_cheby) {
        const double s = chebyshev_step(p.n_cheby, i_cheby);
        // Solver::apply_avc_diff_bcs -> Flow_bc::apply_diffusion (src/Boundary_condition.cpp:43-52)
        #pragma omp parallel for
        for (int i = 0; i < m.n_bc_con; ++i) {
          const int* c = m.bc_con + 4*i;
          const double* in = slot(c[0], false);
          double* gh = slot(c[1], false);
          for (int k2 = 0; k2 < nv*nfq; ++k2) gh[k2] = in[k2];
        }
        compute_smooth_av(s, diff_time, s);
      }
    }
  }

  // Solver::update_art_visc_smoothness (src/Solver.cpp:457-582); returns art_visc_residual
  double update() const
  {
    const double L = p.advect_length;
    // advection velocity: momentum / sqrt(2 rho E) (Solver.cpp:468-478)
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) {
      double* state = k.elem(e);
      for (int q = 0; q < nq; ++q) {
        double scale = std::sqrt(2*state[ND*nq + q]*state[(ND + 1)*nq + q]);
        for (int d = 0; d < ND; ++d) state[d*nq + q] /= scale;
      }
    }
    max_dt_advection();
    for (int iter = 0; iter < p.advect_iters; ++iter) {
      #pragma omp parallel for
      for (int e = 0; e < n_elem(); ++e) write_face_advection(e);
      refine(n_adv_extrap, true, false, false);   // compute_prolong_advection
      for (int i = 0; i < 2; ++i) {
        #pragma omp parallel for
        for (int j = 0; j < m.n_bc_con; ++j) apply_advection_bc(j);
        compute_advection(i);
      }
    }
    // projection onto the Legendre mode of degree av_rs - 1 (Solver.cpp:527-542)
    const double* orth = k.t.ortho + (size_t)(p.av_row_size - 1)*RS;
    #pragma omp parallel for
    for (int e = 0; e < n_elem(); ++e) {
      double* fc = forcing(e);
      const double* a_st = adv(e);
      const double* state = k.elem(e);
      for (int q = 0; q < nq; ++q) {
        double proj = 0;
        for (int i = 0; i < RS; ++i) proj += a_st[i*nq + q]*k.t.weight[i]*orth[i];
        fc[q] = proj*proj*2*state[(ND + 1)*nq + q]/state[ND*nq + q];
      }
    }
    // root-smear-square (Solver.cpp:544-550)
    const int n_real = n_forcing - 1;
    diffuse_art_visc(p.diff_ratio*L*L/n_real);
    // coefficient, residual and the momentum put back (Solver.cpp:552-575)
    const double mult = p.visc_mult*L;
    const double us_max = L*p.unscaled_max*std::sqrt(2*p.freestream_energy/p.freestream_mass);
    double qw[nq];
    for (int q = 0; q < nq; ++q) {
      double w = 1.;
      for (int d = 0; d < ND; ++d) w *= k.t.weight[(q/ipow(RS, ND - 1 - d))%RS];
      qw[q] = w;
    }
    double resid = 0;
    for (int e = 0; e < n_elem(); ++e) {
      double* state = k.elem(e);
      double* av = state + (nv + 1)*nq;
      const double* fc = forcing(e);
      double volume = 1.;
      for (int d = 0; d < ND; ++d) volume *= m.nom_size[e];
      for (int q = 0; q < nq; ++q) {
        double f = mult*fc[n_real*nq + q];
        double new_av = us_max*f/(us_max + f);
        double diff = av[q] - new_av;
        resid += diff*diff*qw[q]*volume;
        av[q] = new_av;
        double scale = std::sqrt(2*state[ND*nq + q]*state[(ND + 1)*nq + q]);
        for (int d = 0; d < ND; ++d) state[d*nq + q] *= scale;
      }
    }
    k.write_face();   // compute_write_face and compute_prolong (Solver.cpp:577-578)
    k.refine(true, false, false);
    return std::sqrt(resid);
  }
};

} // namespace

extern "C" {

// OpenMP threads of the oracle's parallel loops (the reference's hexecute runs
// omp_get_max_threads() - 2, src/hexecute.cpp:7). n <= 0 leaves the count unchanged; returns
// the count in effect.
int oracle_set_threads(int n)
{
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}

int oracle_write_face(const hexed_mesh_desc* m) { return dispatch(m, [](auto& k) { k.write_face(); }); }
int oracle_prolong(const hexed_mesh_desc* m, int scale, int offset)
{ return dispatch(m, [&](auto& k) { k.refine(true, scale, offset); }); }
int oracle_restrict(const hexed_mesh_desc* m, int scale, int offset)
{ return dispatch(m, [&](auto& k) { k.refine(false, scale, offset); }); }
int oracle_apply_state_bcs(const hexed_mesh_desc* m) { return dispatch(m, [](auto& k) { k.apply_state_bcs(); }); }
int oracle_apply_flux_bcs(const hexed_mesh_desc* m) { return dispatch(m, [](auto& k) { k.apply_flux_bcs(); }); }
int oracle_neighbor(const hexed_mesh_desc* m, int viscous) { return dispatch(m, [&](auto& k) { k.neighbor(viscous); }); }
int oracle_compute_euler(const hexed_mesh_desc* m, double dt, int stage, int cr, int uf)
{ return dispatch(m, [&](auto& k) { k.compute_euler(dt, stage, cr, uf); }); }
int oracle_compute_navier_stokes(const hexed_mesh_desc* m, double dt, int stage, int cr, int uf,
                                 const hexed_transport* visc, const hexed_transport* cond)
{ return dispatch(m, [&](auto& k) { k.compute_navier_stokes(dt, stage, cr, uf, *visc, *cond); }); }
int oracle_max_dt(const hexed_mesh_desc* m, double msc, double msd, int local_time, int viscous,
                  const hexed_transport* visc, const hexed_transport* cond, double* out)
{ return dispatch(m, [&](auto& k) { *out = k.max_dt(viscous, msc, msd, local_time, *visc, *cond); }); }
int oracle_set_art_visc_admis(const hexed_mesh_desc* m, double char_speed)
{
  if (!m || m->n_vert <= 0 || !m->vert_id) return HEXED_ERR_INVALID;
  return dispatch(m, [&](auto& k) { k.set_art_visc_admis(char_speed); });
}
int oracle_residual_norm(const hexed_mesh_desc* m, double* out)
{ return dispatch(m, [&](auto& k) { k.residual_norm(out); }); }

// Unit-level entry points for the restated reference tests.
// Derivative::operator() on one row (include/Derivative.hpp:50-55)
int oracle_derivative(int rs, const double* f, const double* fb, double* out)
{
  hexed_mesh_desc m{};
  m.n_dim = 2; m.row_size = rs;
  return dispatch(&m, [&](auto& k) { k.derivative(f, fb, out); });
}

// Face_permutation::match_faces index map (include/Spatial.hpp:85-129)
int oracle_perm_index(int nd, int rs, int dir, int q)
{
  int r = -1;
  hexed_mesh_desc m{};
  m.n_dim = nd; m.row_size = rs;
  dispatch(&m, [&](auto& k) { r = k.perm_index(dir, q); });
  return r;
}

// Characteristics (include/pde.hpp:182-256): eigenvalues [3] and decomposition [nv][3]
int oracle_characteristics(int nd, const double* state, const double* normal, const double* state1,
                           double* eigvals, double* decomp)
{
  hexed_mesh_desc m{};
  m.n_dim = nd; m.row_size = 2;
  return dispatch(&m, [&](auto& k) {
    using KT = std::remove_reference_t<decltype(k)>;
    typename KT::Characteristics ch(state, normal);
    for (int i = 0; i < 3; ++i) eigvals[i] = ch.vals[i];
    double d[KT::nv][3];
    ch.decomp(state1, d);
    for (int r = 0; r < KT::nv; ++r) for (int c = 0; c < 3; ++c) decomp[r*3 + c] = d[r][c];
  });
}

// Solver::update (src/Solver.cpp:834-886); returns the last dt through *out_dt
int oracle_update(const hexed_mesh_desc* m, const hexed_update_params* p, double* out_dt)
{
  int st = HEXED_OK;
  int ds = dispatch(m, [&](auto& k) {
    double dt = 0.;
    for (int i_flow = 0; i_flow < p->flow_iters; ++i_flow) {
      double max_cheby = chebyshev_step(p->n_cheby_flow, p->n_cheby_flow - 1);
      for (int i_cheby = 0; i_cheby < p->n_cheby_flow; ++i_cheby) {
        // Case.cpp:432: set_art_visc_admis before each update when diffusive_admissibility is on
        if (p->av_admis_char_speed > 0 && i_flow == 0 && i_cheby == 0) k.set_art_visc_admis(p->av_admis_char_speed);
        double nominal = std::min(k.max_dt(p->use_ldg, p->max_safety/max_cheby, p->max_safety, p->local_time,
                                           p->visc, p->cond), p->max_time_step);
        dt = nominal*chebyshev_step(p->n_cheby_flow, i_cheby);
        bool fixed = false;
        for (int i = 0; i < 2; ++i) {
          k.apply_state_bcs();
          if (p->use_ldg && !i) k.compute_navier_stokes(dt, i, false, p->use_filter, p->visc, p->cond);
          else k.compute_euler(dt, i, false, p->use_filter);
          if (p->fix_admis) {   // src/Solver.cpp:866-867
            int iters = k.fix_admissibility(*p, p->fix_admis_max_safety, chebyshev_step);
            if (iters < 0) { st = HEXED_ERR_NUMERICAL; return; }
            fixed = iters || fixed;
          }
        }
        if (fixed) break;
      }
    }
    if (out_dt) *out_dt = dt;
  });
  return st != HEXED_OK ? st : ds;
}

// Solver::fix_admissibility (src/Solver.cpp:961-1095)
int oracle_fix_admissibility(const hexed_mesh_desc* m, const hexed_update_params* p, double stability_ratio,
                             int* iterations)
{
  int st = HEXED_OK;
  int ds = dispatch(m, [&](auto& k) {
    const int it = k.fix_admissibility(*p, stability_ratio, chebyshev_step);
    if (it < 0) st = HEXED_ERR_NUMERICAL;
    else *iterations = it;
  });
  return st != HEXED_OK ? st : ds;
}

// Face-slot size (doubles) of the smoothness-AV face storage: max(2*nv, nd + row_size)*nfq
int oracle_sav_slot_dof(int nd, int rs)
{
  int r = -1;
  hexed_mesh_desc m{};
  m.n_dim = nd; m.row_size = rs;
  dispatch(&m, [&](auto& k) {
    using KT = std::remove_reference_t<decltype(k)>;
    r = Sav<KT::n_dim, KT::row_size>::slot_dof;
  });
  return r;
}

// Solver::update_art_visc_smoothness (src/Solver.cpp:457-582). `aux` is
// [n_elem][4 + 2*row_size][nq] (forcing, advection state, its residual cache), `face`
// [n_slot][oracle_sav_slot_dof]; *residual receives art_visc_residual.
int oracle_update_art_visc_smoothness(const hexed_mesh_desc* m, double* aux, double* face,
                                      const oracle_sav_params* p, double* residual)
{
  if (!m || !aux || !face || !p || !residual || !m->vert_tss) return HEXED_ERR_INVALID;
  if (p->av_row_size < 2 || p->av_row_size > m->row_size || !(p->advect_length > 0)) return HEXED_ERR_INVALID;
  return dispatch(m, [&](auto& k) {
    using KT = std::remove_reference_t<decltype(k)>;
    Sav<KT::n_dim, KT::row_size> s(k, aux, face, *p);
    *residual = s.update();
  });
}

// Solver::compute_residual (src/Solver.cpp:899-913)
int oracle_compute_residual(const hexed_mesh_desc* m, const hexed_update_params* p)
{
  return dispatch(m, [&](auto& k) {
    k.apply_state_bcs();
    if (p->use_ldg) k.compute_navier_stokes(1., 0, true, p->use_filter, p->visc, p->cond);
    else k.compute_euler(1., 0, true, p->use_filter);
  });
}

}
