/* kernel_layer_update.c -- a C caller of libhexed_gpu.so that drives Solver::update through
 * the kernel-layer entry points of include/hexed_gpu.h, in the order a reference-side shim
 * sees them when Solver::update (src/Solver.cpp:834-886) keeps its own body:
 *
 *   initialize (src/Solver.cpp:398-407): compute_write_face, compute_prolong
 *   per update, when the AV coefficient is set from the state (Case.cpp:432 before update):
 *     set_art_visc_admis
 *   per flow iteration and Chebyshev sub-step:
 *     max_dt (src/Solver.cpp:122-133) at max_safety / chebyshev_step(n, n - 1), capped at
 *     max_time_step and scaled by chebyshev_step(n, i);
 *     per stage i = 0, 1: apply_state_bcs (src/Solver.cpp:56-67), then compute_navier_stokes
 *     for stage 0 when use_ldg, else compute_euler; then fix_admissibility when it is on.
 *
 * A second context on the same arena runs hexed_gpu_update, the whole update as one call. The
 * program writes every time step and both final element arrays, and exits non-zero (with
 * hexed_gpu_last_error on stderr) if any call fails.
 *
 *   kernel_layer_update <arena file> <output file>
 *
 * Arena file: int32 header[16] = {0x48584431, n_dim, row_size, n_car_elem, n_def_elem, n_slot,
 * n_car_con, n_def_con, n_bc_con, n_ref_face, n_bc_spec, n_vert, n_updates, 0, 0, 0}, one
 * hexed_update_params record, then the arena arrays in hexed_mesh_desc order (elem, rcache,
 * face, nom_size, vert_tss, jac, face_nrml, car_con, def_con, def_con_nrml, bc_con, bc_nrml,
 * bc_cache, ref_face, bc_spec records, vert_id when n_vert > 0).
 * Output file: double dt_kernel_layer[n_updates], dt_update[n_updates], then the element
 * array [n_elem][nv + 3][nq] of the kernel-layer context and of the hexed_gpu_update context.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "hexed_gpu.h"

#define CHECK(call) do { int st_ = (call); if (st_ != HEXED_OK) { \
  fprintf(stderr, "%s failed (%d): %s\n", #call, st_, hexed_gpu_last_error()); exit(2); } } while (0)

static void* read_block(FILE* f, size_t bytes)
{
  void* p = malloc(bytes ? bytes : 1);
  if (!p || fread(p, 1, bytes, f) != bytes) { fprintf(stderr, "arena file truncated\n"); exit(3); }
  return p;
}

/* math::chebyshev_step (src/math.cpp:104-107) */
static double chebyshev_step(int n_steps, int i_step)
{
  const double pi = 3.14159265358979323846;
  return 1./(1. - cos((n_steps - i_step - .5)*pi/n_steps));
}

int main(int argc, char** argv)
{
  if (argc != 3) { fprintf(stderr, "usage: %s arena_file output_file\n", argv[0]); return 1; }
  FILE* f = fopen(argv[1], "rb");
  if (!f) { perror(argv[1]); return 1; }
  int h[16];
  if (fread(h, sizeof(int), 16, f) != 16 || h[0] != 0x48584431) { fprintf(stderr, "not an arena file\n"); return 3; }
  hexed_update_params p;
  if (fread(&p, sizeof p, 1, f) != 1) { fprintf(stderr, "arena file truncated\n"); return 3; }
  hexed_mesh_desc d;
  memset(&d, 0, sizeof d);
  d.n_dim = h[1]; d.row_size = h[2]; d.n_car_elem = h[3]; d.n_def_elem = h[4]; d.n_slot = h[5];
  d.n_car_con = h[6]; d.n_def_con = h[7]; d.n_bc_con = h[8]; d.n_ref_face = h[9]; d.n_bc_spec = h[10];
  d.n_vert = h[11];
  const int n_updates = h[12];
  const size_t nd = (size_t)d.n_dim, nv = nd + 2, nvert = (size_t)1 << nd;
  size_t nq = 1;
  for (size_t i = 0; i < nd; ++i) nq *= (size_t)d.row_size;
  const size_t nfq = nq/(size_t)d.row_size;
  const size_t n_elem = (size_t)d.n_car_elem + (size_t)d.n_def_elem, n_def = (size_t)d.n_def_elem;
  const size_t D = sizeof(double), I = sizeof(int);
  d.elem = read_block(f, n_elem*(nv + 3)*nq*D);
  d.rcache = read_block(f, n_elem*nv*nq*D);
  d.face = read_block(f, (size_t)d.n_slot*2*nv*nfq*D);
  d.nom_size = read_block(f, n_elem*D);
  d.vert_tss = read_block(f, n_elem*nvert*D);
  d.jac = read_block(f, n_def*(nd*nd + 1)*nq*D);
  d.face_nrml = read_block(f, n_def*2*nd*nd*nfq*D);
  d.car_con = read_block(f, (size_t)d.n_car_con*3*I);
  d.def_con = read_block(f, (size_t)d.n_def_con*3*I);
  d.def_con_nrml = read_block(f, (size_t)d.n_def_con*nd*nfq*D);
  d.bc_con = read_block(f, (size_t)d.n_bc_con*4*I);
  d.bc_nrml = read_block(f, (size_t)d.n_bc_con*nd*nfq*D);
  d.bc_cache = read_block(f, (size_t)d.n_bc_con*2*nv*nfq*D);
  d.ref_face = read_block(f, (size_t)d.n_ref_face*7*I);
  d.bc_spec = read_block(f, (size_t)d.n_bc_spec*sizeof(hexed_bc_spec));
  if (d.n_vert > 0) d.vert_id = read_block(f, n_elem*nvert*I);
  fclose(f);

  hexed_gpu_ctx *a = NULL, *b = NULL;
  CHECK(hexed_gpu_create(&d, HEXED_FP64, &a));
  CHECK(hexed_gpu_create(&d, HEXED_FP64, &b));
  hexed_gpu_ctx* both[2] = {a, b};
  for (int k = 0; k < 2; ++k) {   /* Solver::initialize after the state is sampled */
    CHECK(hexed_gpu_compute_write_face(both[k]));
    CHECK(hexed_gpu_compute_prolong(both[k], 0, 0));
  }
  double* dts = calloc((size_t)2*n_updates + 1, D);
  for (int it = 0; it < n_updates; ++it) {
    /* the kernel layer, as Solver::update calls it */
    if (p.av_admis_char_speed > 0) CHECK(hexed_gpu_set_art_visc_admis(a, p.av_admis_char_speed));
    for (int i_flow = 0; i_flow < p.flow_iters; ++i_flow) {
      const int n_cheby = p.n_cheby_flow;
      const double max_cheby = chebyshev_step(n_cheby, n_cheby - 1);
      for (int i_cheby = 0; i_cheby < n_cheby; ++i_cheby) {
        double step = 0.;
        CHECK(hexed_gpu_max_dt(a, p.max_safety/max_cheby, p.max_safety, p.local_time, p.use_filter, p.use_ldg,
                               &p.visc, &p.cond, &step));
        const double dt = (step < p.max_time_step ? step : p.max_time_step)*chebyshev_step(n_cheby, i_cheby);
        int fixed = 0;
        for (int i = 0; i < 2; ++i) {
          CHECK(hexed_gpu_apply_state_bcs(a));
          if (p.use_ldg && !i) CHECK(hexed_gpu_compute_navier_stokes(a, dt, 0, 0, p.use_filter, &p.visc, &p.cond));
          else CHECK(hexed_gpu_compute_euler(a, dt, i, 0, p.use_filter));
          if (p.fix_admis) {
            int iters = 0;
            CHECK(hexed_gpu_fix_admissibility(a, &p, p.fix_admis_max_safety, &iters));
            fixed = fixed || iters > 0;
          }
        }
        dts[it] = dt;
        if (fixed) break;
      }
    }
    /* the same update as one call */
    CHECK(hexed_gpu_update(b, &p, &dts[n_updates + it]));
  }
  const size_t n_out = n_elem*(nv + 3)*nq;
  double* out = malloc(2*n_out*D);
  CHECK(hexed_gpu_download(a, HEXED_ARRAY_ELEM, out));
  CHECK(hexed_gpu_download(b, HEXED_ARRAY_ELEM, out + n_out));
  CHECK(hexed_gpu_destroy(a));
  CHECK(hexed_gpu_destroy(b));
  FILE* g = fopen(argv[2], "wb");
  if (!g) { perror(argv[2]); return 1; }
  if (fwrite(dts, D, (size_t)2*n_updates, g) != (size_t)2*n_updates || fwrite(out, D, 2*n_out, g) != 2*n_out) {
    fprintf(stderr, "short write\n");
    return 4;
  }
  fclose(g);
  printf("kernel_layer_update: %d updates of %zu elements\n", n_updates, n_elem);
  return 0;
}
