// hexed_gpu.cu -- C ABI (include/hexed_gpu.h): context, arena upload, entry points.
//
// Every entry point validates its arguments on the host before anything reaches the
// device: all connection, boundary and refined-face indices of the arena are range
// checked at creation, so no kernel can be handed an out-of-range slot.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdarg>
#include <string>
#include <vector>
#include <algorithm>
#include <mutex>
#include <limits>
#include "ctx.h"
#include "kernels.cuh"
#include "sav.cuh"
#include "basis_tables.h"

using hx::Ctx;

namespace {

thread_local std::string g_error;

int fail(int status, const char* fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return status;
}

#define HX_CUDA(call) do { cudaError_t err_ = (call); if (err_ != cudaSuccess) \
  return fail(err_ == cudaErrorMemoryAllocation ? HEXED_ERR_ALLOC : HEXED_ERR_CUDA, "%s: %s (%s:%d)", #call, \
              cudaGetErrorString(err_), __FILE__, __LINE__); } while (0)

#define HX_LAUNCHED() do { cudaError_t err_ = cudaGetLastError(); if (err_ != cudaSuccess) \
  return fail(HEXED_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(err_)); } while (0)

hx::HostTables host_tables(int rs)
{
  using namespace hexed_tables;
  switch (rs) {
#define HX_T(n) case n: return {node##n, weight##n, diff_mat##n, boundary##n, filter##n, prolong##n, restrict_##n, orthogonal##n, max_cfl##n, min_eig_diffusion##n, step_ratio};
    HX_T(2) HX_T(3) HX_T(4) HX_T(5) HX_T(6) HX_T(7) HX_T(8)
#undef HX_T
  }
  return {};
}

const hx::OpsTable* lookup_ops(int nd, int rs, int precision)
{
  switch (nd*16 + rs) {
    case 2*16 + 2: return hx::ops_2_2(precision);
    case 2*16 + 3: return hx::ops_2_3(precision);
    case 2*16 + 4: return hx::ops_2_4(precision);
    case 2*16 + 5: return hx::ops_2_5(precision);
    case 2*16 + 6: return hx::ops_2_6(precision);
    case 2*16 + 7: return hx::ops_2_7(precision);
    case 2*16 + 8: return hx::ops_2_8(precision);
    case 3*16 + 2: return hx::ops_3_2(precision);
    case 3*16 + 3: return hx::ops_3_3(precision);
    case 3*16 + 4: return hx::ops_3_4(precision);
    case 3*16 + 5: return hx::ops_3_5(precision);
    case 3*16 + 6: return hx::ops_3_6(precision);
    case 3*16 + 7: return hx::ops_3_7(precision);
    case 3*16 + 8: return hx::ops_3_8(precision);
  }
  return nullptr;
}

// chebyshev_step (src/math.cpp:104-107)
double chebyshev_step(int n_steps, int i_step)
{
  return 1/(1 - std::cos((n_steps - i_step - 0.5)*M_PI/n_steps));
}

template <typename T>
int upload_array(T** dst, const T* src, size_t count, const char* name)
{
  *dst = nullptr;
  if (count == 0) return HEXED_OK;
  if (!src) return fail(HEXED_ERR_INVALID, "arena array `%s` is null but %zu entries are required", name, count);
  HX_CUDA(cudaMalloc((void**)dst, count*sizeof(T)));
  HX_CUDA(cudaMemcpy(*dst, src, count*sizeof(T), cudaMemcpyHostToDevice));
  return HEXED_OK;
}

// Scratch-like arena arrays (state, residual cache, traces, BC caches) may be passed as null:
// the device copy then starts at zero.
template <typename T>
int upload_or_zero(T** dst, const T* src, size_t count, const char* name)
{
  if (src || count == 0) return upload_array(dst, src, count, name);
  HX_CUDA(cudaMalloc((void**)dst, count*sizeof(T)));
  HX_CUDA(cudaMemset(*dst, 0, count*sizeof(T)));
  return HEXED_OK;
}

int validate(const hexed_mesh_desc* d)
{
  if (!d) return fail(HEXED_ERR_INVALID, "null mesh descriptor");
  if (d->n_dim < 2 || d->n_dim > 3 || d->row_size < HEXED_MIN_ROW_SIZE || d->row_size > HEXED_MAX_ROW_SIZE)
    return fail(HEXED_ERR_INVALID, "demand for invalid kernel: n_dim %d row_size %d (supported: n_dim 2-3, row_size %d-%d)",
                d->n_dim, d->row_size, HEXED_MIN_ROW_SIZE, HEXED_MAX_ROW_SIZE);
  if (d->n_car_elem < 0 || d->n_def_elem < 0 || d->n_car_con < 0 || d->n_def_con < 0 || d->n_bc_con < 0 ||
      d->n_ref_face < 0 || d->n_bc_spec < 0)
    return fail(HEXED_ERR_INVALID, "negative count in mesh descriptor");
  const long n_elem = (long)d->n_car_elem + d->n_def_elem;
  if (n_elem == 0) return fail(HEXED_ERR_INVALID, "mesh has no elements");
  // the face kernels and Max_dt index face points and points with 32-bit unsigned integers
  long nfq = 1;
  for (int i = 1; i < d->n_dim; ++i) nfq *= d->row_size;
  const long n_con = (long)d->n_car_con + d->n_def_con + d->n_bc_con;
  if (n_con*nfq >= (1L << 31))
    return fail(HEXED_ERR_INVALID, "%ld connections of %ld face points each: over 2^31 face points", n_con, nfq);
  if (n_elem*nfq*d->row_size >= (1L << 31))   // Max_dt indexes quadrature points the same way
    return fail(HEXED_ERR_INVALID, "%ld elements of %ld points each: over 2^31 points", n_elem, nfq*d->row_size);
  if (d->n_slot < n_elem*2*d->n_dim) return fail(HEXED_ERR_INVALID, "n_slot %d < 2*n_dim*n_elem", d->n_slot);
  auto slot_ok = [&](int s) { return s >= 0 && s < d->n_slot; };
  for (int i = 0; i < d->n_car_con; ++i) {
    const int* c = d->car_con + 3*i;
    if (!slot_ok(c[0]) || !slot_ok(c[1]) || c[2] < 0 || c[2] >= d->n_dim)
      return fail(HEXED_ERR_INVALID, "Cartesian connection %d out of range", i);
  }
  for (int i = 0; i < d->n_def_con; ++i) {
    const int* c = d->def_con + 3*i;
    if (!slot_ok(c[0]) || !slot_ok(c[1]) || (c[2] & 3) >= d->n_dim || ((c[2] >> 2) & 3) >= d->n_dim || (c[2] >> 6))
      return fail(HEXED_ERR_INVALID, "deformed connection %d out of range", i);
  }
  for (int i = 0; i < d->n_bc_con; ++i) {
    const int* c = d->bc_con + 4*i;
    if (!slot_ok(c[0]) || !slot_ok(c[1]) || (c[2] & 3) >= d->n_dim || (c[2] >> 3) || c[3] < 0 || c[3] >= d->n_bc_spec)
      return fail(HEXED_ERR_INVALID, "boundary connection %d out of range", i);
  }
  for (int i = 0; i < d->n_bc_spec; ++i)
    if (d->bc_spec[i].kind < 0 || d->bc_spec[i].kind > HEXED_BC_NO_SLIP)
      return fail(HEXED_ERR_INVALID, "boundary condition %d has unknown kind %d", i, d->bc_spec[i].kind);
  if (d->n_vert < 0) return fail(HEXED_ERR_INVALID, "negative vertex count");
  if (d->n_vert > 0) {
    if (!d->vert_id) return fail(HEXED_ERR_INVALID, "n_vert > 0 but no vertex table");
    const long n = n_elem << d->n_dim;
    for (long i = 0; i < n; ++i)
      if (d->vert_id[i] < 0 || d->vert_id[i] >= d->n_vert)
        return fail(HEXED_ERR_INVALID, "vertex id %d of entry %ld out of range", d->vert_id[i], i);
  }
  for (int i = 0; i < d->n_ref_face; ++i) {
    const int* r = d->ref_face + 7*i;
    int nf = 1 << (d->n_dim - 1);
    for (int k = 0; k < d->n_dim - 1; ++k) nf /= 1 + (r[5 + k] != 0);
    if (!slot_ok(r[0])) return fail(HEXED_ERR_INVALID, "refined face %d: coarse slot out of range", i);
    for (int k = 0; k < nf; ++k)
      if (!slot_ok(r[1 + k])) return fail(HEXED_ERR_INVALID, "refined face %d: fine slot %d out of range", i, k);
  }
  return HEXED_OK;
}

size_t array_count(const Ctx* c, int which)
{
  const size_t n_elem = c->cap_car + c->n_def;
  switch (which) {
    case HEXED_ARRAY_ELEM: return n_elem*(c->nv + 3)*c->nq;
    case HEXED_ARRAY_RCACHE: return n_elem*c->nv*c->nq;
    case HEXED_ARRAY_FACE: return (size_t)c->n_slot*2*c->nv*c->nfq;
    case HEXED_ARRAY_BC_CACHE: return (size_t)c->cap_bc_con*2*c->nv*c->nfq;
    case HEXED_ARRAY_NOM_SIZE: return n_elem;
    case HEXED_ARRAY_VERT_TSS: return n_elem << c->nd;
    case HEXED_ARRAY_BC_NRML: return (size_t)c->cap_bc_con*c->nd*c->nfq;
    case HEXED_ARRAY_REF_STATE: return c->ref_state ? n_elem*c->nv : 0;
    case HEXED_ARRAY_JAC: return (size_t)c->n_def*(c->nd*c->nd + 1)*c->nq;
    case HEXED_ARRAY_FACE_NRML: return (size_t)c->n_def*2*c->nd*c->nd*c->nfq;
    case HEXED_ARRAY_DEF_CON_NRML: return (size_t)c->n_def_con*c->nd*c->nfq;
    case HEXED_ARRAY_SAV_AUX: return n_elem*(4 + 2*(size_t)c->rs)*c->nq;
    case HEXED_ARRAY_SAV_FACE: return (size_t)c->n_slot*c->ops->sav_slot_dof();
  }
  return 0;
}

double* array_ptr(Ctx* c, int which)
{
  switch (which) {
    case HEXED_ARRAY_ELEM: return c->elem;
    case HEXED_ARRAY_RCACHE: return c->rcache;
    case HEXED_ARRAY_FACE: return c->face;
    case HEXED_ARRAY_BC_CACHE: return c->bc_cache;
    case HEXED_ARRAY_NOM_SIZE: return c->nom_size;
    case HEXED_ARRAY_VERT_TSS: return c->vert_tss;
    case HEXED_ARRAY_BC_NRML: return c->bc_nrml;
    case HEXED_ARRAY_REF_STATE: return c->ref_state;
    case HEXED_ARRAY_JAC: return c->jac;
    case HEXED_ARRAY_FACE_NRML: return c->face_nrml;
    case HEXED_ARRAY_DEF_CON_NRML: return c->def_con_nrml;
    case HEXED_ARRAY_SAV_AUX: return c->sav_aux;
    case HEXED_ARRAY_SAV_FACE: return c->sav_face;
  }
  return nullptr;
}

// Storage of the smoothness-based AV, allocated on first use: forcing rows and residual cache
// zero, advection state 1 (Solver's constructor, src/Solver.cpp:201-211), face slots zero.
int ensure_sav(Ctx* c)
{
  if (c->sav_aux) return HEXED_OK;
  const size_t n_elem = (size_t)c->cap_car + c->n_def;
  const size_t n_aux = array_count(c, HEXED_ARRAY_SAV_AUX), n_face = array_count(c, HEXED_ARRAY_SAV_FACE);
  double *aux = nullptr, *face = nullptr, *part = nullptr;
  if (cudaMalloc((void**)&aux, n_aux*sizeof(double)) != cudaSuccess ||
      cudaMalloc((void**)&face, n_face*sizeof(double)) != cudaSuccess ||
      cudaMalloc((void**)&part, n_elem*sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    if (aux) cudaFree(aux);
    if (face) cudaFree(face);
    if (part) cudaFree(part);
    return fail(HEXED_ERR_ALLOC, "smoothness-based AV storage allocation failed (%zu + %zu doubles)", n_aux, n_face);
  }
  HX_CUDA(cudaMemsetAsync(aux, 0, n_aux*sizeof(double), c->stream));
  HX_CUDA(cudaMemsetAsync(face, 0, n_face*sizeof(double), c->stream));
  const int n_rows = c->rs, grid = int(std::min<long>(((long)n_elem*n_rows*c->nq + 255)/256, 152*16));
  if (n_elem) hx::k_sav_init<<<grid, 256, 0, c->stream>>>(aux, (long)n_elem, 4 + 2*c->rs, 4, n_rows, (int)c->nq);
  c->sav_aux = aux; c->sav_face = face; c->sav_partials = part;
  HX_LAUNCHED();
  return HEXED_OK;
}

// FP32 device storage of an arena array in the mixed form (face traces, residual cache).
float* f32_array(Ctx* c, int which)
{
  if (c->precision != HEXED_MIXED) return nullptr;
  if (which == HEXED_ARRAY_FACE) return c->face_f;
  if (which == HEXED_ARRAY_RCACHE) return c->rcache_f;
  return nullptr;
}

// After metric data changed on the device: the mixed form's FP32 copies of the normals, and the
// determinant reciprocals.
int refresh_metric_copies(Ctx* c, int which, long offset, long count)
{
  auto narrow = [&](const double* src, float* dst) {
    if (dst && count) hx::k_narrow<<<int(std::min<long>((count + 255)/256, 152*16)), 256, 0, c->stream>>>(
        src + offset, dst + offset, count);
  };
  if (which == HEXED_ARRAY_BC_NRML) narrow(c->bc_nrml, c->bc_nrml_f);
  if (which == HEXED_ARRAY_FACE_NRML) narrow(c->face_nrml, c->face_nrml_f);
  if (which == HEXED_ARRAY_VERT_TSS) narrow(c->vert_tss, c->vert_tss_f);
  if (which == HEXED_ARRAY_DEF_CON_NRML) narrow(c->def_con_nrml, c->def_con_nrml_f);
  if (which == HEXED_ARRAY_REF_STATE) c->ops->ref_terms(*c);
  if (which == HEXED_ARRAY_JAC) {
    narrow(c->jac, c->nrm_f);
    if (c->n_def)
      hx::k_inv_det<<<int(std::min<long>(((long)c->n_def*c->nq + 255)/256, 152*16)), 256, 0, c->stream>>>(
          c->jac, c->inv_det, c->n_def, (int)c->nq, (int)(c->nd*c->nd));
  }
  HX_LAUNCHED();
  return HEXED_OK;
}

// Host <-> device copy of entries [offset, offset + count) of an arena array; FP32-stored
// arrays go through a double staging buffer and a conversion kernel.
int transfer(Ctx* c, int which, long offset, long count, double* host, bool to_device)
{
  const long n = (long)array_count(c, which);
  double* d = array_ptr(c, which);
  float* f = f32_array(c, which);
  if (offset < 0 || count < 0 || offset + count > n || (count && !host))
    return fail(HEXED_ERR_INVALID, "range [%ld, %ld) outside array %d of %ld entries", offset, offset + count, which, n);
  if (count == 0) return HEXED_OK;
  if (which == HEXED_ARRAY_SAV_AUX || which == HEXED_ARRAY_SAV_FACE) {
    if (int st = ensure_sav(c)) return st;
    d = array_ptr(c, which);
  }
  if (!d && !f) return fail(HEXED_ERR_INVALID, "array %d is not allocated", which);
  if (f) {
    double* tmp = nullptr;
    HX_CUDA(cudaMalloc((void**)&tmp, count*sizeof(double)));
    const int grid = int(std::min<long>((count + 255)/256, 152*16));
    cudaError_t err;
    if (to_device) {
      cudaMemcpyAsync(tmp, host, count*sizeof(double), cudaMemcpyHostToDevice, c->stream);
      hx::k_narrow<<<grid, 256, 0, c->stream>>>(tmp, f + offset, count);
    } else {
      hx::k_widen<<<grid, 256, 0, c->stream>>>(f + offset, tmp, count);
      cudaMemcpyAsync(host, tmp, count*sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    }
    err = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (err != cudaSuccess) return fail(HEXED_ERR_CUDA, "transfer: %s", cudaGetErrorString(err));
    return HEXED_OK;
  }
  if (to_device) HX_CUDA(cudaMemcpyAsync(d + offset, host, count*sizeof(double), cudaMemcpyHostToDevice, c->stream));
  else HX_CUDA(cudaMemcpyAsync(host, d + offset, count*sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (to_device) {
    if (int st = refresh_metric_copies(c, which, offset, count)) return st;
  }
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}

// FP32 copy of a device double array (mixed form).
int narrow_copy(Ctx* c, const double* src, float** dst, long n)
{
  *dst = nullptr;
  if (n == 0) return HEXED_OK;
  HX_CUDA(cudaMalloc((void**)dst, n*sizeof(float)));
  hx::k_narrow<<<int(std::min<long>((n + 255)/256, 152*16)), 256, 0, c->stream>>>(src, *dst, n);
  HX_LAUNCHED();
  return HEXED_OK;
}

// Rows of a connection array checked against the arena before upload.
int validate_int_rows(const Ctx* c, int which, const int* rows, long count)
{
  auto slot_ok = [&](int s) { return s >= 0 && s < c->n_slot; };
  for (long i = 0; i < count; ++i) {
    if (which == HEXED_INT_CAR_CON) {
      const int* r = rows + 3*i;
      if (!slot_ok(r[0]) || !slot_ok(r[1]) || r[2] < 0 || r[2] >= c->nd)
        return fail(HEXED_ERR_INVALID, "Cartesian connection row %ld out of range", i);
    } else {
      const int* r = rows + 4*i;
      if (!slot_ok(r[0]) || !slot_ok(r[1]) || (r[2] & 3) >= c->nd || (r[2] >> 3) || r[3] < 0 || r[3] >= c->n_bc_spec)
        return fail(HEXED_ERR_INVALID, "boundary connection row %ld out of range", i);
    }
  }
  return HEXED_OK;
}

int check_ctx(hexed_gpu_ctx* ctx) { return ctx ? HEXED_OK : fail(HEXED_ERR_INVALID, "null context"); }

int set_dt(Ctx* c, double dt)
{
  hx::k_set_scalar<<<1, 1, 0, c->stream>>>(c->scalars, hx::SC_DT, dt);
  HX_LAUNCHED();
  return HEXED_OK;
}

hexed_transport inviscid() { return {0., 0., 1., 1., 0}; }

} // namespace

struct hexed_gpu_ctx : Ctx {};

namespace hx {

ProfScope::ProfScope(Ctx& ctx, const char* name) : c{ctx}, pair{-1}
{
  Profiler* p = c.prof;
  if (!p || !p->enabled || c.capturing || p->n_pairs >= Profiler::max_events/2) return;
  int idx = -1;
  for (int i = 0; i < p->n_names; ++i) if (std::strcmp(p->names[i], name) == 0) { idx = i; break; }
  if (idx < 0) {
    if (p->n_names >= Profiler::max_names) return;
    idx = p->n_names++;
    p->names[idx] = name;
    p->launches[idx] = 0;
    p->total_ms[idx] = 0.;
  }
  pair = p->n_pairs++;
  p->event_name[pair] = idx;
  cudaEventRecord(p->events[2*pair], c.stream);
}

ProfScope::~ProfScope()
{
  if (pair >= 0) cudaEventRecord(c.prof->events[2*pair + 1], c.stream);
}

} // namespace hx

extern "C" {

const char* hexed_gpu_last_error(void) { return g_error.c_str(); }

const char* hexed_gpu_version(void)
{
  static char v[64];
  snprintf(v, sizeof(v), "hexed_gb300 sm_103a n_dim 2-3 row_size %d-%d", HEXED_MIN_ROW_SIZE, HEXED_MAX_ROW_SIZE);
  return v;
}

int hexed_gpu_create(const hexed_mesh_desc* d, int precision, hexed_gpu_ctx** out)
{
  if (!out) return fail(HEXED_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (int st = validate(d)) return st;
  if (precision != HEXED_FP64 && precision != HEXED_MIXED) return fail(HEXED_ERR_INVALID, "unknown precision %d", precision);
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0) {
    cudaGetLastError();
    return fail(HEXED_ERR_NO_DEVICE, "no CUDA device visible");
  }
  hexed_gpu_ctx* c = new hexed_gpu_ctx();
  std::memset(static_cast<Ctx*>(c), 0, sizeof(Ctx));
  c->nd = d->n_dim; c->rs = d->row_size; c->precision = precision;
  HX_CUDA(cudaGetDevice(&c->device));
  c->n_car = d->n_car_elem; c->n_def = d->n_def_elem; c->n_slot = d->n_slot;
  c->n_car_con = d->n_car_con; c->n_def_con = d->n_def_con; c->n_bc_con = d->n_bc_con;
  c->n_ref = d->n_ref_face; c->n_bc_spec = d->n_bc_spec;
  c->cap_car = c->n_car; c->cap_car_con = c->n_car_con; c->cap_bc_con = c->n_bc_con;
  int nq = 1; for (int i = 0; i < c->nd; ++i) nq *= c->rs;
  c->nq = nq; c->nfq = nq/c->rs; c->nv = c->nd + 2;
  c->tables = host_tables(c->rs);
  c->ops = lookup_ops(c->nd, c->rs, precision);
  if (!c->ops) { delete c; return fail(HEXED_ERR_INVALID, "no kernels for n_dim %d row_size %d", d->n_dim, d->row_size); }
  const size_t n_elem = c->n_car + c->n_def;
  const size_t nd = c->nd, nvert = size_t(1) << nd;
  int st = HEXED_OK;
  auto up = [&](auto** dst, const auto* src, size_t n, const char* name) {
    if (st == HEXED_OK) st = upload_array(dst, src, n, name);
  };
  auto up0 = [&](auto** dst, const auto* src, size_t n, const char* name) {
    if (st == HEXED_OK) st = upload_or_zero(dst, src, n, name);
  };
  HX_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  up0(&c->elem, d->elem, n_elem*(c->nv + 3)*c->nq, "elem");
  if (precision == HEXED_FP64) {
    up0(&c->rcache, d->rcache, n_elem*c->nv*c->nq, "rcache");
    up0(&c->face, d->face, (size_t)c->n_slot*2*c->nv*c->nfq, "face");
  } else if (cudaMalloc((void**)&c->rcache_f, n_elem*c->nv*c->nq*sizeof(float)) != cudaSuccess ||
             cudaMalloc((void**)&c->face_f, (size_t)c->n_slot*2*c->nv*c->nfq*sizeof(float)) != cudaSuccess) {
    st = fail(HEXED_ERR_ALLOC, "trace allocation failed");
  } else {
    if (!d->rcache) cudaMemset(c->rcache_f, 0, n_elem*c->nv*c->nq*sizeof(float));
    if (!d->face) cudaMemset(c->face_f, 0, (size_t)c->n_slot*2*c->nv*c->nfq*sizeof(float));
  }
  up(&c->nom_size, d->nom_size, n_elem, "nom_size");
  up(&c->vert_tss, d->vert_tss, n_elem*nvert, "vert_tss");
  up(&c->jac, d->jac, (size_t)c->n_def*(nd*nd + 1)*c->nq, "jac");
  up(&c->face_nrml, d->face_nrml, (size_t)c->n_def*2*nd*nd*c->nfq, "face_nrml");
  up(&c->car_con, d->car_con, (size_t)c->n_car_con*3, "car_con");
  up(&c->def_con, d->def_con, (size_t)c->n_def_con*3, "def_con");
  up(&c->def_con_nrml, d->def_con_nrml, (size_t)c->n_def_con*nd*c->nfq, "def_con_nrml");
  up(&c->bc_con, d->bc_con, (size_t)c->n_bc_con*4, "bc_con");
  up(&c->bc_nrml, d->bc_nrml, (size_t)c->n_bc_con*nd*c->nfq, "bc_nrml");
  up0(&c->bc_cache, d->bc_cache, (size_t)c->n_bc_con*2*c->nv*c->nfq, "bc_cache");
  up(&c->ref_face, d->ref_face, (size_t)c->n_ref*7, "ref_face");
  up(&c->bc_spec, d->bc_spec, (size_t)c->n_bc_spec, "bc_spec");
  c->n_vert = d->n_vert;
  if (c->n_vert > 0) {
    up(&c->vert_id, d->vert_id, n_elem*nvert, "vert_id");
    if (st == HEXED_OK && (cudaMalloc((void**)&c->uncert, n_elem*sizeof(double)) != cudaSuccess ||
                           cudaMalloc((void**)&c->vmax, c->n_vert*sizeof(double)) != cudaSuccess))
      st = fail(HEXED_ERR_ALLOC, "vertex scratch allocation failed");
  }
  if (st != HEXED_OK) { hexed_gpu_destroy(c); return st; }
  if (precision == HEXED_MIXED) {
    // staged FP32 traces and residual cache; FP32 copies of the metric normals
    if (!st && d->rcache) st = transfer(c, HEXED_ARRAY_RCACHE, 0, (long)array_count(c, HEXED_ARRAY_RCACHE), d->rcache, true);
    if (!st && d->face) st = transfer(c, HEXED_ARRAY_FACE, 0, (long)array_count(c, HEXED_ARRAY_FACE), d->face, true);
    if (!st) st = narrow_copy(c, c->jac, &c->nrm_f, (long)c->n_def*(nd*nd + 1)*c->nq);
    if (!st) st = narrow_copy(c, c->face_nrml, &c->face_nrml_f, (long)c->n_def*2*nd*nd*c->nfq);
    if (!st) st = narrow_copy(c, c->def_con_nrml, &c->def_con_nrml_f, (long)c->n_def_con*nd*c->nfq);
    if (!st) st = narrow_copy(c, c->bc_nrml, &c->bc_nrml_f, (long)c->n_bc_con*nd*c->nfq);
    if (!st) st = narrow_copy(c, c->vert_tss, &c->vert_tss_f, (long)n_elem*nvert);
    // reference state of every element: the mean of its own initial state over its quadrature
    // points (zero without one; hexed_gpu_set_reference_state or HEXED_ARRAY_REF_STATE set it
    // then), so that the FP32 offsets carry only the variation inside the element
    std::vector<double> refs(n_elem*c->nv, 0.);
    const size_t nq_ = c->nq, nv_ = c->nv;
    for (size_t e = 0; d->elem && e < n_elem; ++e)
      for (size_t v = 0; v < nv_; ++v) {
        double sum = 0.;
        for (size_t q = 0; q < nq_; ++q) sum += d->elem[(e*(nv_ + 3) + v)*nq_ + q];
        refs[e*nv_ + v] = sum/double(nq_);
      }
    if (!st) st = upload_array(&c->ref_state, refs.data(), refs.size(), "reference state");
    if (!st && cudaMalloc((void**)&c->ref_terms, n_elem*((3*nd + 7 + 3)/4*4)*sizeof(float)) != cudaSuccess)
      st = fail(HEXED_ERR_ALLOC, "reference-term allocation failed");
    if (!st) c->ops->ref_terms(*c);
    // owners of the slots beyond the element slots: boundary ghosts take the inside element,
    // hanging-face mortars the coarse element
    const size_t elem_slots = n_elem*2*nd;
    std::vector<int> owner(c->n_slot > (int)elem_slots ? c->n_slot - elem_slots : 1, 0);
    for (int i = 0; i < c->n_bc_con; ++i) {
      const int* r = d->bc_con + 4*i;
      if (r[1] >= (int)elem_slots) owner[r[1] - elem_slots] = r[0]/int(2*nd);
    }
    for (int i = 0; i < c->n_ref; ++i) {
      const int* r = d->ref_face + 7*i;
      int n_fine = 1 << (nd - 1);
      for (size_t k = 0; k + 1 < nd; ++k) n_fine /= 1 + (r[5 + k] != 0);
      for (int k = 1; k <= n_fine; ++k) if (r[k] >= (int)elem_slots) owner[r[k] - elem_slots] = r[0]/int(2*nd);
    }
    if (!st) st = upload_array(&c->slot_elem, owner.data(), owner.size(), "slot owners");
  }
  if (!st && c->n_def) {
    if (cudaMalloc((void**)&c->inv_det, (size_t)c->n_def*c->nq*sizeof(double)) != cudaSuccess) {
      st = fail(HEXED_ERR_ALLOC, "determinant allocation failed");
    } else {
      hx::k_inv_det<<<int(std::min<long>(((long)c->n_def*c->nq + 255)/256, 152*16)), 256, 0, c->stream>>>(
          c->jac, c->inv_det, c->n_def, (int)c->nq, (int)(nd*nd));
    }
  }
  if (st != HEXED_OK) { hexed_gpu_destroy(c); return st; }
  c->local_variant = 0;
  c->face_threads = 256;
  c->max_partials = 152*16*8;
  if (cudaMalloc((void**)&c->partials, c->max_partials*sizeof(double)) != cudaSuccess ||
      cudaMalloc((void**)&c->record, n_elem*sizeof(int)) != cudaSuccess ||
      cudaMalloc((void**)&c->scalars, hx::SC_N*sizeof(double)) != cudaSuccess ||
      cudaMalloc((void**)&c->status, 4*sizeof(int)) != cudaSuccess ||
      cudaMalloc((void**)&c->dt_ticket, sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc((void**)&c->d_norm, 4*sizeof(double)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_pinned, 8*sizeof(double)) != cudaSuccess) {
    hexed_gpu_destroy(c);
    return fail(HEXED_ERR_ALLOC, "scratch allocation failed");
  }
  cudaMemset(c->scalars, 0, hx::SC_N*sizeof(double));
  cudaMemset(c->status, 0, 4*sizeof(int));
  cudaMemset(c->dt_ticket, 0, sizeof(unsigned));
  HX_CUDA(cudaDeviceSynchronize());
  *out = c;
  return HEXED_OK;
}

int hexed_gpu_destroy(hexed_gpu_ctx* c)
{
  if (!c) return HEXED_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* ptrs[] = {c->elem, c->rcache, c->face, c->nom_size, c->vert_tss, c->jac, c->face_nrml, c->car_con,
                  c->def_con, c->def_con_nrml, c->bc_con, c->bc_nrml, c->bc_cache, c->ref_face, c->bc_spec,
                  c->scalars, c->partials, c->status, c->dt_ticket, c->d_norm, c->vert_id, c->uncert, c->vmax,
                  c->seg_table, c->seg_out, c->inv_det, c->face_f, c->rcache_f, c->nrm_f, c->face_nrml_f,
                  c->def_con_nrml_f, c->bc_nrml_f, c->vert_tss_f, c->ref_state, c->ref_terms, c->record, c->slot_elem,
                  c->state_stage,
                  c->sav_aux, c->sav_face, c->sav_partials};
  for (void* p : ptrs) if (p) cudaFree(p);
  if (c->graph) {
    if (c->graph->exec) cudaGraphExecDestroy(c->graph->exec);
    delete c->graph;
  }
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  if (c->prof) {
    if (c->prof->created) for (auto& e : c->prof->events) cudaEventDestroy(e);
    delete c->prof;
  }
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return HEXED_OK;
}

int hexed_gpu_upload(hexed_gpu_ctx* c, int which, const double* host)
{
  if (int st = check_ctx(c)) return st;
  return transfer(c, which, 0, (long)array_count(c, which), const_cast<double*>(host), true);
}

int hexed_gpu_download(hexed_gpu_ctx* c, int which, double* host)
{
  if (int st = check_ctx(c)) return st;
  return transfer(c, which, 0, (long)array_count(c, which), host, false);
}

int hexed_gpu_synchronize(hexed_gpu_ctx* c)
{
  if (int st = check_ctx(c)) return st;
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}

int hexed_gpu_compute_euler(hexed_gpu_ctx* c, double dt, int i_stage, int compute_residual, int use_filter)
{
  if (int st = check_ctx(c)) return st;
  if (i_stage && compute_residual)
    return fail(HEXED_ERR_PRECONDITION, "residual calculation is a single-stage operation");
  if (int st = set_dt(c, dt)) return st;
  c->ops->compute_euler(*c, i_stage ? 1 : 0, compute_residual, use_filter, false, hx::LocalDt{0, 0., 0., 0.});
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_compute_navier_stokes(hexed_gpu_ctx* c, double dt, int i_stage, int compute_residual, int use_filter,
                                    const hexed_transport* visc, const hexed_transport* cond)
{
  if (int st = check_ctx(c)) return st;
  if (!visc || !cond) return fail(HEXED_ERR_INVALID, "null transport model");
  if (i_stage) return fail(HEXED_ERR_PRECONDITION, "two-stage stabilization is not applicable to diffusion equations");
  if (int st = set_dt(c, dt)) return st;
  c->ops->compute_navier_stokes(*c, 0, compute_residual, use_filter, *visc, *cond, false);
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_max_dt(hexed_gpu_ctx* c, double msc, double msd, int local_time, int use_filter, int viscous,
                     const hexed_transport* visc, const hexed_transport* cond, double* out_dt)
{
  (void)use_filter;
  if (int st = check_ctx(c)) return st;
  hexed_transport inv = inviscid();
  c->ops->max_dt(*c, msc, msd, local_time, viscous, visc ? *visc : inv, cond ? *cond : inv,
                 1.7976931348623157e308, 1.);
  HX_LAUNCHED();
  if (out_dt) {
    HX_CUDA(cudaMemcpyAsync(c->h_pinned, c->scalars + hx::SC_MAXDT, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    HX_CUDA(cudaStreamSynchronize(c->stream));
    *out_dt = c->h_pinned[0];
  }
  return HEXED_OK;
}

int hexed_gpu_compute_prolong(hexed_gpu_ctx* c, int scale, int offset)
{
  if (int st = check_ctx(c)) return st;
  c->ops->refine(*c, true, scale, offset);
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_compute_restrict(hexed_gpu_ctx* c, int scale, int offset)
{
  if (int st = check_ctx(c)) return st;
  c->ops->refine(*c, false, scale, offset);
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_compute_write_face(hexed_gpu_ctx* c)
{
  if (int st = check_ctx(c)) return st;
  c->ops->write_face(*c, 0, c->n_car + c->n_def);
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_compute_jacobian(hexed_gpu_ctx* c, const double* vert_pos)
{
  if (int st = check_ctx(c)) return st;
  if (c->n_def && !vert_pos) return fail(HEXED_ERR_INVALID, "null vertex positions");
  const size_t nvert = size_t(1) << c->nd;
  const size_t n_pos = (size_t)c->n_def*nvert*c->nd, n_fn = (size_t)c->n_def*2*c->nd*c->nd*c->nfq,
               n_vt = (size_t)c->n_def*nvert;
  double* scratch = nullptr;
  if (c->n_def) {
    HX_CUDA(cudaMalloc((void**)&scratch, (n_pos + n_fn + n_vt)*sizeof(double)));
    cudaError_t err = cudaMemcpyAsync(scratch, vert_pos, n_pos*sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (err != cudaSuccess) { cudaFree(scratch); return fail(HEXED_ERR_CUDA, "%s", cudaGetErrorString(err)); }
  }
  c->ops->compute_jacobian(*c, scratch, scratch + n_pos, scratch + n_pos + n_fn);
  cudaError_t err = cudaGetLastError();
  int st = HEXED_OK;
  if (err != cudaSuccess) st = fail(HEXED_ERR_CUDA, "metric kernels: %s", cudaGetErrorString(err));
  const long n_jac = (long)array_count(c, HEXED_ARRAY_JAC), n_fnr = (long)array_count(c, HEXED_ARRAY_FACE_NRML),
             n_con = (long)array_count(c, HEXED_ARRAY_DEF_CON_NRML), n_bc = (long)array_count(c, HEXED_ARRAY_BC_NRML);
  if (!st) st = refresh_metric_copies(c, HEXED_ARRAY_JAC, 0, n_jac);
  if (!st) st = refresh_metric_copies(c, HEXED_ARRAY_FACE_NRML, 0, n_fnr);
  if (!st) st = refresh_metric_copies(c, HEXED_ARRAY_DEF_CON_NRML, 0, n_con);
  if (!st) st = refresh_metric_copies(c, HEXED_ARRAY_BC_NRML, 0, n_bc);
  if (!st) st = refresh_metric_copies(c, HEXED_ARRAY_VERT_TSS, 0, (long)array_count(c, HEXED_ARRAY_VERT_TSS));
  err = cudaStreamSynchronize(c->stream);
  if (scratch) cudaFree(scratch);
  if (!st && err != cudaSuccess) st = fail(HEXED_ERR_CUDA, "metric set-up: %s", cudaGetErrorString(err));
  return st;
}

int hexed_gpu_is_admissible(hexed_gpu_ctx* c, int* admissible, int* record)
{
  if (int st = check_ctx(c)) return st;
  if (!admissible) return fail(HEXED_ERR_INVALID, "null output");
  c->ops->admissible(*c, c->record);
  HX_LAUNCHED();
  HX_CUDA(cudaMemcpyAsync(c->h_pinned, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (record)
    HX_CUDA(cudaMemcpyAsync(record, c->record, (size_t)(c->n_car + c->n_def)*sizeof(int), cudaMemcpyDeviceToHost,
                            c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  int flags;
  std::memcpy(&flags, c->h_pinned, sizeof(int));
  *admissible = !(flags & 1);
  if (flags & 2) return fail(HEXED_ERR_NUMERICAL, "state is not finite");
  return HEXED_OK;
}

int hexed_gpu_device_flags(hexed_gpu_ctx* c, int* flags)
{
  if (int st = check_ctx(c)) return st;
  if (!flags) return fail(HEXED_ERR_INVALID, "null output");
  HX_CUDA(cudaMemcpyAsync(c->h_pinned, c->status + 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  std::memcpy(flags, c->h_pinned, sizeof(int));
  return HEXED_OK;
}

int hexed_gpu_check_conversions(const double* host, long n, long* mismatches)
{
  if (!mismatches || n < 0 || (n && !host)) return fail(HEXED_ERR_INVALID, "bad arguments");
  *mismatches = 0;
  if (n == 0) return HEXED_OK;
  double* d_in = nullptr;
  unsigned long long* d_count = nullptr;
  HX_CUDA(cudaMalloc((void**)&d_in, n*sizeof(double)));
  if (cudaMalloc((void**)&d_count, sizeof(unsigned long long)) != cudaSuccess) {
    cudaFree(d_in);
    return fail(HEXED_ERR_ALLOC, "allocation failed");
  }
  unsigned long long count = 0;
  cudaError_t err = cudaMemcpy(d_in, host, n*sizeof(double), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(d_count, 0, sizeof(unsigned long long));
  if (err == cudaSuccess) {
    hx::k_check_conversions<<<int(std::min<long>((n + 255)/256, 152*16)), 256>>>(d_in, n, d_count);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpy(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost);
  cudaFree(d_in);
  cudaFree(d_count);
  if (err != cudaSuccess) return fail(HEXED_ERR_CUDA, "conversion check: %s", cudaGetErrorString(err));
  *mismatches = (long)count;
  return HEXED_OK;
}

int hexed_gpu_set_launch_shape(hexed_gpu_ctx* c, int local_variant, int face_threads)
{
  if (int st = check_ctx(c)) return st;
  if (local_variant < 0 || local_variant > 2) return fail(HEXED_ERR_INVALID, "launch-shape variant %d not in 0..2", local_variant);
  if (local_variant && c->nd == 3) return fail(HEXED_ERR_INVALID, "3D volume kernels have one launch shape");
  if (face_threads != 64 && face_threads != 128 && face_threads != 256)
    return fail(HEXED_ERR_INVALID, "face kernels take 64, 128 or 256 threads per CTA, not %d", face_threads);
  HX_CUDA(cudaStreamSynchronize(c->stream));
  c->local_variant = local_variant;
  c->face_threads = face_threads;
  if (c->graph) c->graph->valid = false;   // the captured launches used the previous shape
  return HEXED_OK;
}

int hexed_gpu_launch_shape(hexed_gpu_ctx* c, int* local_elems_per_cta, int* face_threads)
{
  if (int st = check_ctx(c)) return st;
  if (local_elems_per_cta) *local_elems_per_cta = c->ops->local_elems_per_cta(c->local_variant);
  if (face_threads) *face_threads = c->face_threads;
  return HEXED_OK;
}

int hexed_gpu_set_reference_state(hexed_gpu_ctx* c, const double* state)
{
  if (int st = check_ctx(c)) return st;
  if (!state) return fail(HEXED_ERR_INVALID, "null reference state");
  for (size_t v = 0; v < c->nv; ++v)
    if (!std::isfinite(state[v])) return fail(HEXED_ERR_INVALID, "non-finite reference state");
  if (!(state[c->nd] > 0)) return fail(HEXED_ERR_INVALID, "reference density must be positive");
  if (c->precision != HEXED_MIXED) return HEXED_OK;
  const size_t n = (size_t)c->cap_car + c->n_def;
  std::vector<double> refs(n*c->nv);
  for (size_t e = 0; e < n; ++e)
    for (size_t v = 0; v < c->nv; ++v) refs[e*c->nv + v] = state[v];
  HX_CUDA(cudaMemcpyAsync(c->ref_state, refs.data(), refs.size()*sizeof(double), cudaMemcpyHostToDevice, c->stream));
  c->ops->ref_terms(*c);
  HX_LAUNCHED();
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}

int hexed_gpu_write_face_range(hexed_gpu_ctx* c, int elem_begin, int elem_count)
{
  if (int st = check_ctx(c)) return st;
  if (elem_begin < 0 || elem_count < 0 || (long)elem_begin + elem_count > (long)c->cap_car + c->n_def)
    return fail(HEXED_ERR_INVALID, "elements [%d, %ld) outside the arena", elem_begin, (long)elem_begin + elem_count);
  c->ops->write_face(*c, elem_begin, elem_count);
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_set_art_visc_admis(hexed_gpu_ctx* c, double char_speed)
{
  if (int st = check_ctx(c)) return st;
  if (c->n_vert <= 0) return fail(HEXED_ERR_INVALID, "set_art_visc_admis needs the arena's vertex table");
  c->ops->set_art_visc_admis(*c, char_speed);
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_update_art_visc_smoothness(hexed_gpu_ctx* c, const hexed_sav_params* p, double* residual)
{
  if (int st = check_ctx(c)) return st;
  if (!p) return fail(HEXED_ERR_INVALID, "null smoothness-AV parameters");
  if (!(p->advect_length > 0) || !std::isfinite(p->advect_length))
    return fail(HEXED_ERR_INVALID, "advect_length must be positive and finite");
  if (p->advect_iters < 0 || p->diff_iters < 0 || p->n_cheby < 1)
    return fail(HEXED_ERR_INVALID, "iteration counts must be >= 0 and n_cheby >= 1");
  // Solver::set_art_visc_row_size (src/Solver.cpp:660-665)
  if (p->av_row_size < 2 || p->av_row_size > c->rs)
    return fail(HEXED_ERR_PRECONDITION, "`row_size` must be >= 2 and <= discretization row size");
  if (!(p->advect_safety > 0) || !(p->diff_safety > 0) || !(p->diff_ratio > 0) || !(p->unscaled_max > 0) ||
      !(p->freestream_mass > 0) || !(p->freestream_energy > 0))
    return fail(HEXED_ERR_INVALID, "safety factors, diff_ratio, unscaled_max and the freestream must be positive");
  if (int st = ensure_sav(c)) return st;
  c->ops->update_art_visc_smoothness(*c, *p, c->d_norm + 3);
  HX_LAUNCHED();
  if (residual) {
    HX_CUDA(cudaMemcpyAsync(c->h_pinned, c->d_norm + 3, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    HX_CUDA(cudaStreamSynchronize(c->stream));
    *residual = c->h_pinned[0];
  }
  return HEXED_OK;
}

int hexed_gpu_apply_state_bcs(hexed_gpu_ctx* c)
{
  if (int st = check_ctx(c)) return st;
  c->ops->bc_state(*c);
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_apply_flux_bcs(hexed_gpu_ctx* c)
{
  if (int st = check_ctx(c)) return st;
  c->ops->bc_flux(*c);
  HX_LAUNCHED();
  return HEXED_OK;
}

namespace {
// Solver::is_admissible on the device, read back to the host (synchronizes the stream)
int admissible_now(Ctx* c, bool* admissible)
{
  c->ops->admissible(*c, c->record);
  HX_LAUNCHED();
  HX_CUDA(cudaMemcpyAsync(c->h_pinned, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  int flags;
  std::memcpy(&flags, c->h_pinned, sizeof(int));
  if (flags & 2) return fail(HEXED_ERR_NUMERICAL, "state is not finite");
  *admissible = !(flags & 1);
  return HEXED_OK;
}

// The diffusion of one Solver::fix_admissibility iteration (src/Solver.cpp:985-1089), after
// its admissibility check: the coefficient set-up and bulk/Laplacian swap, the local Max_dt of
// pde::Fix_therm_admis, two Fix_therm_admis sub-steps of the LDG chain (state BC fused into
// the boundary Neighbor: ghost = inside), the flow's Max_dt of the fixed state, and the swap
// back. The flow's step and raw max_dt (scalars[0, 2)) are kept across it, as the reference's
// stage keeps its opts.dt.
int fix_iteration(Ctx* c, const hexed_update_params* p, double stability_ratio)
{
  const hexed_transport inv = inviscid();
  c->ops->fix_admis_coef(*c, c->record, false);
  hx::k_copy_scalars<<<1, 32, 0, c->stream>>>(c->scalars, hx::SC_DT, hx::SC_SAVED, 2);
  c->fta = 1;
  c->ops->max_dt(*c, stability_ratio, stability_ratio, 1, 1, inv, inv, std::numeric_limits<double>::max(), 1.);
  // dt = 1 split into two sub-steps (src/Solver.cpp:1060-1064)
  const double linear = 1., quadratic = 1./8/0.9;
  double step[2];
  step[1] = (linear + std::sqrt(linear*linear - 4*quadratic))/2.;
  step[0] = quadratic/step[1];
  for (double s : step) {
    if (int st = set_dt(c, s)) { c->fta = 0; return st; }
    c->ops->compute_navier_stokes(*c, 0, 0, 0, inv, inv, true);
  }
  c->fta = 0;
  const double max_cheby = chebyshev_step(p->n_cheby_flow, p->n_cheby_flow - 1);
  c->ops->max_dt(*c, p->max_safety/max_cheby, p->max_safety, p->local_time, p->use_ldg, p->visc, p->cond,
                 p->max_time_step, 1.);
  hx::k_copy_scalars<<<1, 32, 0, c->stream>>>(c->scalars, hx::SC_SAVED, hx::SC_DT, 2);
  c->ops->fix_admis_coef(*c, nullptr, true);
  HX_LAUNCHED();
  return HEXED_OK;
}

// Solver::fix_admissibility (src/Solver.cpp:961-1095): *iters as the reference returns it
int fix_admissibility(Ctx* c, const hexed_update_params* p, double stability_ratio, int* iters)
{
  if (c->n_vert > 0 && !c->uncert) return fail(HEXED_ERR_INVALID, "vertex scratch missing");
  int iter;
  int n_iters = std::numeric_limits<int>::max();
  for (iter = 0; iter < n_iters; ++iter) {
    if (iter >= 100000) return fail(HEXED_ERR_NUMERICAL, "failed to fix thermodynamic admissability in %i iterations", iter);
    bool adm;
    if (int st = admissible_now(c, &adm)) return st;
    if (adm) {
      if (iter) n_iters = std::min(n_iters, 2*iter);
      else {
        ++iter;
        break;
      }
    } else {
      n_iters = std::numeric_limits<int>::max();
    }
    if (int st = fix_iteration(c, p, stability_ratio)) return st;
  }
  --iter;
  *iters = iter;
  return HEXED_OK;
}

// Enqueues one Solver::update (src/Solver.cpp:834-886) on the context's stream. With local
// time stepping and no diffusion the step is known on the host (the global part is 1, times
// max_time_step and the Chebyshev factor, as k_max_dt's last CTA would give): the first stage's
// volume kernel then computes each point's time-step scale itself (LocalDt mode 1) instead
// of a separate Max_dt pass, with the same arithmetic, and *host_dt receives the step.
// Otherwise *host_dt is NaN and the step stays on the device.
int enqueue_update(hexed_gpu_ctx* c, const hexed_update_params* p, double* host_dt = nullptr)
{
  if (host_dt) *host_dt = std::nan("");
  if (p->av_admis_char_speed > 0) {
    // Case.cpp:432: set_art_visc_admis before the update when diffusive_admissibility is on
    if (c->n_vert <= 0) return fail(HEXED_ERR_INVALID, "artificial viscosity needs the arena's vertex table");
    c->ops->set_art_visc_admis(*c, p->av_admis_char_speed);
  }
  const bool fuse_dt = p->local_time && !p->use_ldg && !p->fix_admis;
  const double max_cheby = chebyshev_step(p->n_cheby_flow, p->n_cheby_flow - 1);
  for (int i_flow = 0; i_flow < p->flow_iters; ++i_flow) {
    for (int i_cheby = 0; i_cheby < p->n_cheby_flow; ++i_cheby) {
      const double msc = p->max_safety/max_cheby, msd = p->max_safety;
      const double cheby = chebyshev_step(p->n_cheby_flow, i_cheby);
      if (fuse_dt) {
        const double dt = std::fmin(1., p->max_time_step)*cheby;
        const double icc = hx::inv_cfl_conv(*c, msc), icd = hx::inv_cfl_diff(*c, msd);
        c->ops->compute_euler(*c, 0, 0, p->use_filter, true, hx::LocalDt{1, icc, icd, dt});
        c->ops->compute_euler(*c, 1, 0, p->use_filter, true, hx::LocalDt{2, icc, icd, dt});
        if (host_dt) *host_dt = dt;
        continue;
      }
      c->ops->max_dt(*c, msc, msd, p->local_time, p->use_ldg, p->visc, p->cond, p->max_time_step, cheby);
      bool fixed = false;
      for (int i = 0; i < 2; ++i) {
        if (p->use_ldg && !i) c->ops->compute_navier_stokes(*c, 0, 0, p->use_filter, p->visc, p->cond, true);
        else c->ops->compute_euler(*c, i, 0, p->use_filter, true, hx::LocalDt{0, 0., 0., 0.});
        if (p->fix_admis) {
          // Solver.cpp:866-867: every stage ends with fix_admissibility; a fixed update
          // leaves the Chebyshev loop after its two stages
          int iters = 0;
          if (int st = fix_admissibility(c, p, p->fix_admis_max_safety, &iters)) return st;
          fixed = iters || fixed;
        }
      }
      if (fixed) break;
    }
  }
  return HEXED_OK;
}

bool same_params(const hexed_update_params& a, const hexed_update_params& b)
{
  return std::memcmp(&a, &b, sizeof(a)) == 0;
}
} // namespace

int hexed_gpu_fix_admissibility(hexed_gpu_ctx* c, const hexed_update_params* p, double stability_ratio, int* iterations)
{
  if (int st = check_ctx(c)) return st;
  if (!p || !iterations || p->n_cheby_flow < 1 || !(stability_ratio > 0))
    return fail(HEXED_ERR_INVALID, "bad fix_admissibility arguments");
  return fix_admissibility(c, p, stability_ratio, iterations);
}

int hexed_gpu_update_n(hexed_gpu_ctx* c, const hexed_update_params* p, int n, int use_graph)
{
  if (int st = check_ctx(c)) return st;
  if (!p || p->n_cheby_flow < 1 || p->flow_iters < 0 || n < 0) return fail(HEXED_ERR_INVALID, "bad update parameters");
  if (!use_graph || p->fix_admis) {   // the admissibility fix reads back to the host: eager
    for (int i = 0; i < n; ++i) if (int st = enqueue_update(c, p)) return st;
    HX_LAUNCHED();
    return HEXED_OK;
  }
  if (!c->graph) c->graph = new hx::GraphCache();
  hx::GraphCache& g = *c->graph;
  if (!(g.valid && g.n == n && same_params(g.params, *p) && g.n_car == c->n_car && g.n_car_con == c->n_car_con &&
        g.n_bc_con == c->n_bc_con)) {
    if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    g.valid = false;
    // one eager update first so every kernel's attributes are set outside the capture
    if (int st = enqueue_update(c, p)) return st;
    HX_CUDA(cudaStreamSynchronize(c->stream));
    cudaGraph_t graph = nullptr;
    HX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    int st = HEXED_OK;
    for (int i = 0; i < n && st == HEXED_OK; ++i) st = enqueue_update(c, p);
    c->capturing = false;
    cudaError_t err = cudaStreamEndCapture(c->stream, &graph);
    if (st != HEXED_OK) { if (graph) cudaGraphDestroy(graph); return st; }
    if (err != cudaSuccess) return fail(HEXED_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(err));
    err = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (err != cudaSuccess) return fail(HEXED_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(err));
    g.valid = true; g.n = n; g.params = *p; g.n_car = c->n_car; g.n_car_con = c->n_car_con; g.n_bc_con = c->n_bc_con;
    n -= 1;   // the eager update above counts
    if (n == 0) return HEXED_OK;
    // replay the graph for the remaining updates in whole multiples, the rest eagerly
    for (int i = 0; i < n % g.n; ++i) if (int s2 = enqueue_update(c, p)) return s2;
    for (int i = 0; i < n/g.n; ++i) HX_CUDA(cudaGraphLaunch(g.exec, c->stream));
    HX_LAUNCHED();
    return HEXED_OK;
  }
  HX_CUDA(cudaGraphLaunch(g.exec, c->stream));
  return HEXED_OK;
}

int hexed_gpu_write_range(hexed_gpu_ctx* c, int which, long offset, long count, const double* host)
{
  if (int st = check_ctx(c)) return st;
  return transfer(c, which, offset, count, const_cast<double*>(host), true);
}

int hexed_gpu_read_range(hexed_gpu_ctx* c, int which, long offset, long count, double* host)
{
  if (int st = check_ctx(c)) return st;
  return transfer(c, which, offset, count, host, false);
}

namespace {
// Conserved state rows of the active elements, host [n][nv][nq] <-> device elem rows 0..nv-1,
// on the context's stream: in, one contiguous copy to a staging buffer and a scatter kernel;
// out, one strided (2D) copy. (Splitting a copy over several copy streams was measured and
// changed nothing: the host link runs at ~209 GB/s in and ~191 GB/s out on this part.)
int state_copy(Ctx* c, double* host, bool to_device)
{
  if (!host) return fail(HEXED_ERR_INVALID, "null state buffer");
  const size_t n = (size_t)c->n_car + c->n_def;
  if (n == 0) return HEXED_OK;
  const size_t width = c->nv*c->nq*sizeof(double), pitch = (c->nv + 3)*c->nq*sizeof(double);
  if (to_device) {
    // one contiguous transfer into a staging buffer, then a scatter kernel: measured on this
    // part at 209 GB/s against 150 GB/s for the strided (2D) host-to-device copy
    if (!c->state_stage && cudaMalloc((void**)&c->state_stage, n*width) != cudaSuccess) {
      cudaGetLastError();
      c->state_stage = nullptr;
    }
    if (c->state_stage) {
      HX_CUDA(cudaMemcpyAsync(c->state_stage, host, n*width, cudaMemcpyHostToDevice, c->stream));
      const long total = (long)n*c->nv*c->nq;
      hx::k_scatter_rows<<<int(std::min<long>((total + 255)/256, 152*16)), 256, 0, c->stream>>>(
          c->state_stage, c->elem, (long)n, int(c->nv*c->nq), int((c->nv + 3)*c->nq));
      HX_LAUNCHED();
    } else {
      HX_CUDA(cudaMemcpy2DAsync(c->elem, pitch, host, width, width, n, cudaMemcpyHostToDevice, c->stream));
    }
  } else {
    // the strided device-to-host copy already runs at the link's rate (190 GB/s)
    HX_CUDA(cudaMemcpy2DAsync(host, width, c->elem, pitch, width, n, cudaMemcpyDeviceToHost, c->stream));
  }
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}
} // namespace

int hexed_gpu_write_state(hexed_gpu_ctx* c, const double* state)
{
  if (int st = check_ctx(c)) return st;
  return state_copy(c, const_cast<double*>(state), true);
}

int hexed_gpu_read_state(hexed_gpu_ctx* c, double* state)
{
  if (int st = check_ctx(c)) return st;
  return state_copy(c, state, false);
}

int hexed_gpu_write_int_range(hexed_gpu_ctx* c, int which, long offset, long count, const int* host)
{
  if (int st = check_ctx(c)) return st;
  const int width = which == HEXED_INT_CAR_CON ? 3 : which == HEXED_INT_BC_CON ? 4 : 0;
  const long rows = which == HEXED_INT_CAR_CON ? c->cap_car_con : c->cap_bc_con;
  int* dst = which == HEXED_INT_CAR_CON ? c->car_con : c->bc_con;
  if (!width || offset < 0 || count < 0 || offset + count > rows || (count && !host))
    return fail(HEXED_ERR_INVALID, "rows [%ld, %ld) outside int array %d of %ld rows", offset, offset + count, which, rows);
  if (int st = validate_int_rows(c, which, host, count)) return st;
  if (count) HX_CUDA(cudaMemcpyAsync(dst + offset*width, host, count*width*sizeof(int), cudaMemcpyHostToDevice, c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}

int hexed_gpu_write_bc_spec(hexed_gpu_ctx* c, int index, const hexed_bc_spec* spec)
{
  if (int st = check_ctx(c)) return st;
  if (!spec || index < 0 || index >= c->n_bc_spec) return fail(HEXED_ERR_INVALID, "bad boundary-condition index %d", index);
  if (spec->kind < 0 || spec->kind > HEXED_BC_NO_SLIP) return fail(HEXED_ERR_INVALID, "unknown BC kind %d", spec->kind);
  HX_CUDA(cudaMemcpyAsync(c->bc_spec + index, spec, sizeof(*spec), cudaMemcpyHostToDevice, c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}

int hexed_gpu_set_active(hexed_gpu_ctx* c, int n_car_elem, int n_car_con, int n_bc_con)
{
  if (int st = check_ctx(c)) return st;
  if (c->n_def) return fail(HEXED_ERR_INVALID, "set_active applies to Cartesian-only arenas");
  if (n_car_elem < 0 || n_car_elem > c->cap_car || n_car_con < 0 || n_car_con > c->cap_car_con || n_bc_con < 0 ||
      n_bc_con > c->cap_bc_con)
    return fail(HEXED_ERR_INVALID, "active sizes exceed the arena");
  c->n_car = n_car_elem; c->n_car_con = n_car_con; c->n_bc_con = n_bc_con;
  return HEXED_OK;
}

int hexed_gpu_segment_residual_norms(hexed_gpu_ctx* c, int n_seg, const int* elem_begin, const int* elem_count,
                                     double* out)
{
  if (int st = check_ctx(c)) return st;
  if (n_seg < 0 || (n_seg && (!elem_begin || !elem_count || !out))) return fail(HEXED_ERR_INVALID, "bad segment table");
  if (n_seg == 0) return HEXED_OK;
  for (int i = 0; i < n_seg; ++i)
    if (elem_begin[i] < 0 || elem_count[i] < 1 || (long)elem_begin[i] + elem_count[i] > (long)c->n_car + c->n_def)
      return fail(HEXED_ERR_INVALID, "segment %d outside the active elements", i);
  if (n_seg > c->seg_capacity) {
    if (c->seg_table) cudaFree(c->seg_table);
    if (c->seg_out) cudaFree(c->seg_out);
    c->seg_table = nullptr; c->seg_out = nullptr; c->seg_capacity = 0;
    HX_CUDA(cudaMalloc((void**)&c->seg_table, 2*n_seg*sizeof(int)));
    HX_CUDA(cudaMalloc((void**)&c->seg_out, 3*n_seg*sizeof(double)));
    c->seg_capacity = n_seg;
  }
  HX_CUDA(cudaMemcpyAsync(c->seg_table, elem_begin, n_seg*sizeof(int), cudaMemcpyHostToDevice, c->stream));
  HX_CUDA(cudaMemcpyAsync(c->seg_table + n_seg, elem_count, n_seg*sizeof(int), cudaMemcpyHostToDevice, c->stream));
  c->ops->segment_residual_norms(*c, n_seg, c->seg_table, c->seg_table + n_seg, c->seg_out);
  HX_LAUNCHED();
  HX_CUDA(cudaMemcpyAsync(out, c->seg_out, 3*n_seg*sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}

int hexed_gpu_update(hexed_gpu_ctx* c, const hexed_update_params* p, double* out_dt)
{
  if (int st = check_ctx(c)) return st;
  if (!p || p->n_cheby_flow < 1 || p->flow_iters < 0) return fail(HEXED_ERR_INVALID, "bad update parameters");
  double host_dt;
  if (int st = enqueue_update(c, p, &host_dt)) return st;
  HX_LAUNCHED();
  if (out_dt) {
    if (!std::isnan(host_dt)) {
      *out_dt = host_dt;
    } else {
      HX_CUDA(cudaMemcpyAsync(c->h_pinned, c->scalars + hx::SC_DT, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      HX_CUDA(cudaStreamSynchronize(c->stream));
      *out_dt = c->h_pinned[0];
    }
  }
  return HEXED_OK;
}

int hexed_gpu_compute_residual(hexed_gpu_ctx* c, const hexed_update_params* p)
{
  if (int st = check_ctx(c)) return st;
  if (!p) return fail(HEXED_ERR_INVALID, "null parameters");
  if (int st = set_dt(c, 1.)) return st;
  if (p->use_ldg) c->ops->compute_navier_stokes(*c, 0, 1, p->use_filter, p->visc, p->cond, true);
  else c->ops->compute_euler(*c, 0, 1, p->use_filter, true, hx::LocalDt{0, 0., 0., 0.});
  HX_LAUNCHED();
  return HEXED_OK;
}

int hexed_gpu_residual_norm(hexed_gpu_ctx* c, double out[3])
{
  if (int st = check_ctx(c)) return st;
  if (!out) return fail(HEXED_ERR_INVALID, "null output");
  c->ops->residual_norm(*c, c->d_norm);
  HX_LAUNCHED();
  HX_CUDA(cudaMemcpyAsync(c->h_pinned, c->d_norm, 3*sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < 3; ++i) out[i] = c->h_pinned[i];
  return HEXED_OK;
}

void* hexed_gpu_stream(hexed_gpu_ctx* c) { return c ? (void*)c->stream : nullptr; }

int hexed_gpu_fp64_peak(double* tflops)
{
  if (!tflops) return fail(HEXED_ERR_INVALID, "null output");
  int dev = 0, n_sm = 0;
  HX_CUDA(cudaGetDevice(&dev));
  HX_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  double* out = nullptr;
  const int block = 256, blocks = n_sm*8, iters = 4096;
  HX_CUDA(cudaMalloc((void**)&out, (size_t)blocks*block*sizeof(double)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  hx::k_fp64_fma<<<blocks, block>>>(out, iters, 1.0000001);   // warm-up
  cudaEventRecord(e0);
  hx::k_fp64_fma<<<blocks, block>>>(out, iters, 1.0000001);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return fail(HEXED_ERR_CUDA, "fp64 probe: %s", cudaGetErrorString(err));
  *tflops = 2.*hx::fp64_fma_chains*double(iters)*blocks*block/(ms*1e-3)/1e12;
  return HEXED_OK;
}

int hexed_gpu_profile_enable(hexed_gpu_ctx* c, int enable)
{
  if (int st = check_ctx(c)) return st;
  if (!c->prof) c->prof = new hx::Profiler();
  hx::Profiler* p = c->prof;
  if (!p->created) {
    for (auto& e : p->events) HX_CUDA(cudaEventCreate(&e));
    p->created = true;
  }
  HX_CUDA(cudaStreamSynchronize(c->stream));
  p->enabled = enable != 0;
  p->n_pairs = 0;
  p->n_names = 0;
  return HEXED_OK;
}

int hexed_gpu_profile_read(hexed_gpu_ctx* c, hexed_kernel_time* out, int capacity, int* n_out)
{
  if (int st = check_ctx(c)) return st;
  if (n_out) *n_out = 0;
  hx::Profiler* p = c->prof;
  if (!p) return HEXED_OK;
  HX_CUDA(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < p->n_names; ++i) { p->launches[i] = 0; p->total_ms[i] = 0.; }
  for (int k = 0; k < p->n_pairs; ++k) {
    float ms = 0.f;
    HX_CUDA(cudaEventElapsedTime(&ms, p->events[2*k], p->events[2*k + 1]));
    p->launches[p->event_name[k]] += 1;
    p->total_ms[p->event_name[k]] += ms;
  }
  int n = 0;
  for (int i = 0; i < p->n_names && n < capacity; ++i, ++n) {
    std::snprintf(out[n].name, sizeof(out[n].name), "%s", p->names[i]);
    out[n].launches = p->launches[i];
    out[n].total_ms = p->total_ms[i];
  }
  if (n_out) *n_out = n;
  p->n_pairs = 0;
  p->n_names = 0;
  return HEXED_OK;
}

} // extern "C"

// ------------------------------------------------------------------ no-allocation variant
namespace {

// Scratch of hexed_gpu_segment_residual_norms_static, in module memory that exists from load
// time: the norms of up to HEXED_STATIC_MAX_SEGMENTS segments (3 doubles each), then the
// segment table (begins, then counts, as ints packed two to a double slot). Nothing in it has
// to start at zero: every call copies its table in and the kernel writes every norm it returns.
constexpr int static_max_seg = HEXED_STATIC_MAX_SEGMENTS;
static __device__ __align__(256) double g_seg_scratch[3*static_max_seg + static_max_seg];

constexpr int max_devices = 64;
std::mutex g_seg_scratch_lock;
double* g_seg_scratch_addr[max_devices] = {};

// Device address of g_seg_scratch on `device`, looked up once per device with that device
// current (the host-side symbol is not a device address).
int seg_scratch_on(int device, double** out)
{
  if (device < 0 || device >= max_devices) return fail(HEXED_ERR_INVALID, "device %d out of range", device);
  std::lock_guard<std::mutex> guard(g_seg_scratch_lock);
  if (!g_seg_scratch_addr[device]) {
    int current = -1;
    HX_CUDA(cudaGetDevice(&current));
    if (current != device) HX_CUDA(cudaSetDevice(device));
    void* addr = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&addr, g_seg_scratch);
    if (current != device) HX_CUDA(cudaSetDevice(current));
    if (err != cudaSuccess || !addr)
      return fail(HEXED_ERR_CUDA, "cudaGetSymbolAddress of the segment-norm scratch: %s", cudaGetErrorString(err));
    g_seg_scratch_addr[device] = static_cast<double*>(addr);
  }
  *out = g_seg_scratch_addr[device];
  return HEXED_OK;
}

} // namespace

extern "C" int hexed_gpu_segment_residual_norms_static(hexed_gpu_ctx* c, int n_seg, const int* elem_begin,
                                                       const int* elem_count, double* out)
{
  if (int st = check_ctx(c)) return st;
  if (n_seg < 0 || (n_seg && (!elem_begin || !elem_count || !out))) return fail(HEXED_ERR_INVALID, "bad segment table");
  if (n_seg > static_max_seg)
    return fail(HEXED_ERR_INVALID, "%d segments exceed the fixed scratch of this entry point (at most %d)", n_seg,
                static_max_seg);
  for (int i = 0; i < n_seg; ++i)
    if (elem_begin[i] < 0 || elem_count[i] < 1 || (long)elem_begin[i] + elem_count[i] > (long)c->n_car + c->n_def)
      return fail(HEXED_ERR_INVALID, "segment %d outside the active elements", i);
  double* scratch = nullptr;
  if (int st = seg_scratch_on(c->device, &scratch)) return st;
  if (n_seg == 0) return HEXED_OK;
  double* d_out = scratch;
  int* d_table = reinterpret_cast<int*>(scratch + 3*static_max_seg);
  HX_CUDA(cudaMemcpyAsync(d_table, elem_begin, n_seg*sizeof(int), cudaMemcpyHostToDevice, c->stream));
  HX_CUDA(cudaMemcpyAsync(d_table + static_max_seg, elem_count, n_seg*sizeof(int), cudaMemcpyHostToDevice,
                          c->stream));
  c->ops->segment_residual_norms(*c, n_seg, d_table, d_table + static_max_seg, d_out);
  HX_LAUNCHED();
  HX_CUDA(cudaMemcpyAsync(out, d_out, 3*n_seg*sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  HX_CUDA(cudaStreamSynchronize(c->stream));
  return HEXED_OK;
}
