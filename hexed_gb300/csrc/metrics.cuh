// metrics.cuh -- metric set-up of deformed elements on the device: Deformed_element::
// set_jacobian (src/Deformed_element.cpp:15-134) for every deformed element, then the
// connection-level part of Solver::calc_jacobian (src/Solver.cpp:273-381): shared normals of
// deformed connections, boundary normals and the vertex time-step scale shared over vertices.
// Conforming meshes only: the arenas hold hanging faces between Cartesian elements alone,
// which need no normals.
#pragma once
#include "kernels.cuh"

namespace hx {

template <int ND>
__device__ __forceinline__ double det_nd(const double (&a)[ND][ND])
{
  if constexpr (ND == 2) return a[0][0]*a[1][1] - a[0][1]*a[1][0];
  else return a[0][0]*(a[1][1]*a[2][2] - a[1][2]*a[2][1]) - a[0][1]*(a[1][0]*a[2][2] - a[1][2]*a[2][0])
            + a[0][2]*(a[1][0]*a[2][1] - a[1][1]*a[2][0]);
}

// det of `a` with column `col` replaced by the unit vector e_row: the cofactor (row, col)
template <int ND>
__device__ __forceinline__ double cofactor(const double (&a)[ND][ND], int row, int col)
{
  double m[ND][ND];
  #pragma unroll
  for (int i = 0; i < ND; ++i)
    #pragma unroll
    for (int j = 0; j < ND; ++j) m[i][j] = j == col ? (i == row ? 1. : 0.) : a[i][j];
  return det_nd<ND>(m);
}

template <int ND, int RS>
struct MetricSmem {
  static constexpr int nq = ipow(RS, ND);
  // positions [nd][nq], Jacobian [nd][nd][nq], normals and determinant [nd*nd + 1][nq]
  static constexpr size_t bytes = sizeof(double)*(size_t)(ND + ND*ND + ND*ND + 1)*nq;
};

// One CTA per deformed element, one thread per quadrature point. vert_pos [n_def][nvert][nd]
// (vertex bit d <-> reference dim d, dim 0 most significant). Writes jac [n_def][nd*nd+1][nq]
// (reference-level normals [i][j] then det), the element's own face normals
// fn [n_def][2nd][nd][nfq], and its vertex time-step scale vtss [n_def][nvert].
template <int ND, int RS>
__global__ void k_set_jacobian(const double* vert_pos, const double* nom_size, Tab<RS> tab, double* jac, double* fn,
                               double* vtss)
{
  using S = Shape<ND, RS>;
  constexpr int nq = S::nq, nfq = S::nfq, nvert = S::nvert;
  extern __shared__ __align__(16) double s_met[];
  double* s_pos = s_met;                    // [nd][nq]
  double* s_jac = s_pos + ND*nq;            // [nd][nd][nq]
  double* s_nrm = s_jac + ND*ND*nq;         // [nd*nd + 1][nq]
  const int ed = blockIdx.x, q = threadIdx.x;
  const double* vp = vert_pos + (size_t)ed*nvert*ND;
  const double h = nom_size[ed];
  int node[ND];
  #pragma unroll
  for (int d = 0; d < ND; ++d) node[d] = (q/S::stride(d))%RS;
  // position (Deformed_element::position): multilinear in the vertices, last dim contracted first
  if (q < nq) {
    #pragma unroll
    for (int i = 0; i < ND; ++i) {
      double v[nvert];
      #pragma unroll
      for (int b = 0; b < nvert; ++b) v[b] = vp[b*ND + i];
      #pragma unroll
      for (int j = ND - 1; j >= 0; --j) {
        const double xi = tab.node[node[j]];
        const int bit = 1 << (ND - 1 - j);
        #pragma unroll
        for (int b = 0; b < nvert; ++b)
          if (!(b & bit)) v[b] = v[b]*(1. - xi) + v[b | bit]*xi;
      }
      s_pos[i*nq + q] = v[0];
    }
  }
  __syncthreads();
  // Jacobian d pos_i / d ref_j, divided by the nominal size
  double J[ND][ND];
  if (q < nq) {
    #pragma unroll
    for (int i = 0; i < ND; ++i)
      #pragma unroll
      for (int j = 0; j < ND; ++j) {
        const int stride = S::stride(j);
        const double* row = s_pos + i*nq + (q - node[j]*stride);
        double acc = 0.;
        #pragma unroll
        for (int k = 0; k < RS; ++k) acc += tab.diff[node[j]*RS + k]*row[k*stride];
        J[i][j] = acc/h;
        s_jac[(i*ND + j)*nq + q] = J[i][j];
      }
    const double det = det_nd<ND>(J);
    double* out = jac + (size_t)ed*(ND*ND + 1)*nq;
    #pragma unroll
    for (int i = 0; i < ND; ++i)
      #pragma unroll
      for (int j = 0; j < ND; ++j) {
        const double c = cofactor<ND>(J, j, i);
        out[(i*ND + j)*nq + q] = c;
        s_nrm[(i*ND + j)*nq + q] = c;
      }
    out[ND*ND*nq + q] = det;
    s_nrm[ND*ND*nq + q] = det;
  }
  __syncthreads();
  // face normals (src/Deformed_element.cpp:88-116): the Jacobian extrapolated to the face,
  // then the cofactors of the face's own reference dimension
  for (int t = q; t < 2*ND*nfq; t += blockDim.x) {
    const int face = t/nfq, r = t%nfq, i_dim = face/2, sign = face%2;
    const int stride = S::stride(i_dim);
    const int base = (r/stride)*stride*RS + r%stride;
    double F[ND][ND];
    #pragma unroll
    for (int i = 0; i < ND; ++i)
      #pragma unroll
      for (int j = 0; j < ND; ++j) {
        double acc = 0.;
        for (int k = 0; k < RS; ++k) acc += tab.bound[sign*RS + k]*s_jac[(i*ND + j)*nq + base + k*stride];
        F[i][j] = acc;
      }
    for (int j = 0; j < ND; ++j) fn[(((size_t)ed*2*ND + face)*ND + j)*nfq + r] = cofactor<ND>(F, j, i_dim);
  }
  // vertex time-step scale (src/Deformed_element.cpp:117-134): normals and determinant
  // extrapolated to each vertex (B along every dimension), nominal size * det / sum_i |n_i|
  for (int b = q; b < nvert; b += blockDim.x) {
    double vals[ND*ND + 1];
    for (int k = 0; k < ND*ND + 1; ++k) {
      double acc = 0.;
      for (int p = 0; p < nq; ++p) {
        double w = 1.;
        for (int d = 0; d < ND; ++d) w *= tab.bound[((b >> (ND - 1 - d)) & 1)*RS + (p/S::stride(d))%RS];
        acc += w*s_nrm[k*nq + p];
      }
      vals[k] = acc;
    }
    double norm_sum = 0.;
    for (int i = 0; i < ND; ++i) {
      double sq = 0.;
      for (int j = 0; j < ND; ++j) sq += vals[i*ND + j]*vals[i*ND + j];
      norm_sum += sqrt(sq);
    }
    vtss[(size_t)ed*nvert + b] = h*vals[ND*ND]/norm_sum;
  }
}

// Face normals of deformed elements before the connections are known: identity rows, which is
// what a face in a Cartesian connection sees (include/Spatial.hpp:331-339).
template <int ND, int RS>
__global__ void k_identity_face_normals(double* face_nrml, int n_def)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  const long total = (long)n_def*2*ND*ND*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int j = int((t/nfq)%ND), face = int((t/(nfq*ND))%(2*ND));
    face_nrml[t] = j == face/2 ? 1. : 0.;
  }
}

// Shared normal of each deformed connection (src/Solver.cpp:327-352): the average of the two
// element normals with their flip signs, face 1 read through the face permutation; both
// elements' face normals and the connection normal take it (face-0 order for the connection).
template <int ND, int RS>
__global__ void k_def_con_normals(const int* def_con, int n_def_con, int n_car, const double* fn, double* face_nrml,
                                  double* con_nrml)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  const long total = (long)n_def_con*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int i = int(t/nfq), q = int(t%nfq);
    const int* c = def_con + 3*i;
    const int dir = c[2];
    const int f0 = c[0]%(2*ND), f1 = c[1]%(2*ND);
    const int e0 = c[0]/(2*ND) - n_car, e1 = c[1]/(2*ND) - n_car;
    const double s0 = 1 - 2*(((dir >> 4) & 1) == 0), s1 = 1 - 2*(((dir >> 5) & 1) == 1);
    const int q1 = perm_index<ND, RS>(dir, q);
    for (int d = 0; d < ND; ++d) {
      const double n0 = fn[(((size_t)e0*2*ND + f0)*ND + d)*nfq + q];
      const double n1 = fn[(((size_t)e1*2*ND + f1)*ND + d)*nfq + q1];
      const double n = .5*s0*n0 + .5*s1*n1;
      face_nrml[(((size_t)e0*2*ND + f0)*ND + d)*nfq + q] = s0*n;
      face_nrml[(((size_t)e1*2*ND + f1)*ND + d)*nfq + q1] = s1*n;
      con_nrml[((size_t)i*ND + d)*nfq + q] = s0*n;
    }
  }
}

// Boundary normals: the inside element's own face normal for a deformed element (also its
// face normal in the arena), the unit vector of the face's dimension for a Cartesian one.
template <int ND, int RS>
__global__ void k_bc_normals(const int* bc_con, int n_bc, int n_car, const double* fn, double* face_nrml,
                             double* bc_nrml)
{
  constexpr int nfq = Shape<ND, RS>::nfq;
  const long total = (long)n_bc*nfq;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int i = int(t/nfq), q = int(t%nfq);
    const int* c = bc_con + 4*i;
    const int e = c[0]/(2*ND) - n_car, face = c[0]%(2*ND), i_dim = c[2] & 3;
    for (int d = 0; d < ND; ++d) {
      double n;
      if (e >= 0) {
        n = fn[(((size_t)e*2*ND + face)*ND + d)*nfq + q];
        face_nrml[(((size_t)e*2*ND + face)*ND + d)*nfq + q] = n;
      } else {
        n = d == i_dim ? 1. : 0.;
      }
      bc_nrml[((size_t)i*ND + d)*nfq + q] = n;
    }
  }
}

// Vertex time-step scale of every element before sharing: nominal size / nd for Cartesian
// elements (src/Element.cpp:17), the set_jacobian value for deformed ones.
template <int ND>
__global__ void k_element_vtss(const double* nom_size, int n_car, int n_elem, const double* vtss_def, double* vert_tss)
{
  constexpr int nvert = 1 << ND;
  const long total = (long)n_elem*nvert;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x) {
    const int e = int(t/nvert);
    vert_tss[t] = e < n_car ? nom_size[e]/ND : vtss_def[t - (long)n_car*nvert];
  }
}

// share_vertex_data with Vertex::vector_min (src/Solver.cpp:35-54): minimum over the elements
// sharing a vertex, through the IEEE bit patterns of the non-negative values.
static __global__ void k_vertex_min_init(double* vmin, int n_vert)
{
  for (int i = blockIdx.x*blockDim.x + threadIdx.x; i < n_vert; i += gridDim.x*blockDim.x)
    vmin[i] = 1.7976931348623157e308;
}

template <int ND>
__global__ void k_vertex_min(const int* vert_id, int n_elem, const double* vert_tss, double* vmin)
{
  constexpr int nvert = 1 << ND;
  const long total = (long)n_elem*nvert;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x)
    atomicMin(reinterpret_cast<unsigned long long*>(vmin + vert_id[t]),
              (unsigned long long)__double_as_longlong(vert_tss[t]));
}

template <int ND>
__global__ void k_vertex_gather(const int* vert_id, int n_elem, const double* vmin, double* vert_tss)
{
  constexpr int nvert = 1 << ND;
  const long total = (long)n_elem*nvert;
  for (long t = blockIdx.x*(long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x*blockDim.x)
    vert_tss[t] = vmin[vert_id[t]];
}

} // namespace hx
