/*
 * A plain C caller of libmacgpu.so (no Python): SPC/E water built from
 * arrays the way a cook shim flattens molec[]/spec[] (one species, sites O,
 * H, H, three SHAKE constraints per molecule), then
 *   mg_create -> mg_forces (measure) -> mg_md_set_state -> mg_md_steps ->
 *   mg_md_get_state -> mg_destroy.
 *
 * usage: spce_abi IN OUT
 *   IN  (binary doubles): nmol, L, cutoff, alpha, kappa, h, epsc, omegac,
 *       precision (0 FP64, 1 mixed), then r [9 nmol] (forces are evaluated
 *       here), r0 [9 nmol] and r1 [9 nmol] (the MD state to advance one step)
 *   OUT (binary doubles): f [9 nmol], el, lj, r after the step [9 nmol]
 * Exit status 0 on success; every library error is printed.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "macgpu.h"

/* cook program units (sim/units.h:101-108): charge e*408.779826922048,
   energy K (kcal/mol * 4184/8.31446261815324), mass g/mol/0.831446261815324 */
#define ELECTRON 408.779826922048
#define KCAL_K (4184.0 / 8.31446261815324)
#define MUNIT 0.831446261815324

static int check(int rc, mg_ctx *ctx, const char *what) {
  if (rc) fprintf(stderr, "%s failed (%d): %s\n", what, rc, ctx ? mg_last_error(ctx) : "");
  return rc;
}

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: spce_abi IN OUT\n");
    return 2;
  }
  FILE *fi = fopen(argv[1], "rb");
  if (!fi) return 2;
  double hd[9];
  if (fread(hd, sizeof(double), 9, fi) != 9) return 2;
  const int nmol = (int)hd[0], ns = 3 * nmol, nc = 3 * nmol;
  double *r = malloc(sizeof(double) * 3 * ns), *r0 = malloc(sizeof(double) * 3 * ns),
         *r1 = malloc(sizeof(double) * 3 * ns), *f = malloc(sizeof(double) * 3 * ns);
  if (fread(r, sizeof(double), 3 * ns, fi) != (size_t)(3 * ns) ||
      fread(r0, sizeof(double), 3 * ns, fi) != (size_t)(3 * ns) ||
      fread(r1, sizeof(double), 3 * ns, fi) != (size_t)(3 * ns))
    return 2;
  fclose(fi);

  /* the species table: site types 0 = H, 1 = O (EvdW, RvdW as the .ble
     holds them: kcal/mol and A, 12 significant digits) */
  const double type_E[2] = {0.0, -0.155401529637 * KCAL_K};
  const double type_R[2] = {0.5, 1.77685742247};
  const double type_A[2] = {0.0, 0.0};
  const int st[3] = {1, 0, 0};
  const double q[3] = {-0.8476 * ELECTRON, 0.4238 * ELECTRON, 0.4238 * ELECTRON};
  const double m[3] = {15.9994 / MUNIT, 1.008 / MUNIT, 1.008 / MUNIT};
  const int pair[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  const double blen[3] = {1.0, 1.0, sqrt(8.0 / 3.0)}; /* O-H, O-H, H-H (tetrahedral) */

  /* flatten: molecule starts, per-site type/charge/mass, global constraint
     pairs (what the shim builds from molec[n].sp and spec[sp]->si[]) */
  int *mol_first = malloc(sizeof(int) * (nmol + 1)), *mol_cfirst = malloc(sizeof(int) * (nmol + 1));
  int *type = malloc(sizeof(int) * ns), *cons = malloc(sizeof(int) * 2 * nc);
  double *charge = malloc(sizeof(double) * ns), *mass = malloc(sizeof(double) * ns);
  double *clen = malloc(sizeof(double) * nc);
  for (int n = 0; n < nmol; n++) {
    mol_first[n] = 3 * n;
    mol_cfirst[n] = 3 * n;
    for (int i = 0; i < 3; i++) {
      type[3 * n + i] = st[i];
      charge[3 * n + i] = q[i];
      mass[3 * n + i] = m[i];
    }
    for (int a = 0; a < 3; a++) {
      cons[2 * (3 * n + a)] = 3 * n + pair[a][0];
      cons[2 * (3 * n + a) + 1] = 3 * n + pair[a][1];
      clen[3 * n + a] = blen[a];
    }
  }
  mol_first[nmol] = ns;
  mol_cfirst[nmol] = nc;

  mg_topology t = {0};
  t.ns = ns;
  t.nmol = nmol;
  t.mol_first = mol_first;
  t.site_type = type;
  t.charge = charge;
  t.mass = mass;
  t.ntypes = 2;
  t.type_EvdW = type_E;
  t.type_RvdW = type_R;
  t.type_alpha = type_A;
  t.comb_rule = 0;
  t.nc = nc;
  t.cons = cons;
  t.cons_len = clen;
  t.mol_cfirst = mol_cfirst;

  mg_params p = {0};
  p.L[0] = p.L[1] = p.L[2] = hd[1];
  p.cutoff = hd[2];
  p.LJcutoff = hd[2];
  p.alpha = hd[3];
  p.kappa = hd[4];
  p.grid = 256;
  p.rshift = 3;
  p.rplus = 2.5;
  p.epsinf = 3e33;
  p.precision = (int)hd[8];
  p.h = hd[5];
  p.epsc = hd[6];
  p.omegac = hd[7];

  int st_create = 0;
  mg_ctx *ctx = mg_create(&t, &p, &st_create);
  if (!ctx) {
    fprintf(stderr, "mg_create failed (%d)\n", st_create);
    return 1;
  }
  mg_energy e;
  if (check(mg_forces(ctx, r, f, 1, &e), ctx, "mg_forces")) return 1;
  if (check(mg_md_set_state(ctx, r0, r1), ctx, "mg_md_set_state")) return 1;
  if (check(mg_md_steps(ctx, 1, NULL), ctx, "mg_md_steps")) return 1;
  if (check(mg_md_get_state(ctx, r0, r1), ctx, "mg_md_get_state")) return 1;
  if (check(mg_destroy(ctx), NULL, "mg_destroy")) return 1;

  FILE *fo = fopen(argv[2], "wb");
  if (!fo) return 2;
  fwrite(f, sizeof(double), 3 * ns, fo);
  fwrite(&e.el, sizeof(double), 1, fo);
  fwrite(&e.lj, sizeof(double), 1, fo);
  fwrite(r0, sizeof(double), 3 * ns, fo);
  fclose(fo);
  printf("spce_abi: %d molecules, el %.10g lj %.10g\n", nmol, e.el, e.lj);
  return 0;
}
