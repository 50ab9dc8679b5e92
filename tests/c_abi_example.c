/*
 * A plain C caller of the FAME C ABI (include/fame.h): the core of what a MEX
 * gateway or any other foreign-function binding does for the woodpile band
 * problem of band_structure_woodpile_Lanczos_n60_gamma0p2.m.
 *
 *   geometry  fame_rasterize        (Material_Locate_Isofunction.m, woodpile_isofun.m)
 *   material  fame_material_blocks  (Physical_settings_woodpile.m:91-96,184-194)
 *   set-up    fame_plan_create      (SVD_Matrix_Generate.m, Funhand_Generate_Lanzcos.m)
 *   solve     fame_lanczos          (Lanczos.m with op_A, op_B, op_invB)
 *
 * usage: c_abi_example N K   -> prints the K eigenvalues of B^{-1}A at the X
 * point (theta = (pi, 0, pi)), one per line, then the max NFSEP residual.
 *
 * usage: c_abi_example grad N K -> the backward entry on a field-mode plan:
 *   set-up    fame_plan_create_field  eps(r) = 1 + 12 s(r), gamma(r) = 0.2 s(r),
 *                                      s = ((73 i1 + 151 i2 + 37 i3 + 11) mod 97) / 96
 *                                      (no symmetry, so no degenerate bands)
 *   solve     fame_lanczos (FP64), K Ritz vectors kept on the device
 *   backward  fame_eig_gradient of omega_3 - omega_2 (the gap of bands 2, 3)
 * and prints the K frequencies omega = 1/lambda, then "g eps gamma" for every
 * vertex (x fastest).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "fame.h"

static int check(int rc, fame_plan_t plan, const char* what) {
  if (rc != FAME_OK) fprintf(stderr, "%s failed (%d): %s\n", what, rc, fame_last_error(plan));
  return rc;
}

/* 6x6 constitutive block [eps xi; zeta mu] = [e*I, i*g*I; -i*g*I, I], interleaved complex */
static void bi_isotropic(double e, double g, double c6[72]) {
  memset(c6, 0, 72 * sizeof(double));
  for (int d = 0; d < 3; ++d) {
    c6[2 * (d * 6 + d)] = e;                  /* eps */
    c6[2 * ((d + 3) * 6 + d + 3)] = 1.0;      /* mu */
    c6[2 * (d * 6 + d + 3) + 1] = g;          /* xi = +i g */
    c6[2 * ((d + 3) * 6 + d) + 1] = -g;       /* zeta = -i g */
  }
}

static int run_grad(int n, int k) {
  const double pi = 3.14159265358979323846;
  const double lattice[9] = {0.0, 0.5, 0.5, 0.5, 0.0, 0.5, 0.5, 0.5, 0.0};
  const double theta[3] = {pi, 0.0, pi};
  const size_t nq = (size_t)n * n * n, len = 4 * nq;
  double* eps = malloc(sizeof(double) * nq);
  double* gam = malloc(sizeof(double) * nq);
  double* g_host = malloc(sizeof(double) * 2 * nq);
  double* ew = malloc(sizeof(double) * k);
  double* om = malloc(sizeof(double) * k);
  double* w = malloc(sizeof(double) * k);
  void* ev = NULL;
  double* g_dev = NULL;
  fame_plan_t plan = NULL;
  int rc = 0;
  if (!eps || !gam || !g_host || !ew || !om || !w || k < 3) return 1;
  for (int i3 = 0; i3 < n; ++i3)
    for (int i2 = 0; i2 < n; ++i2)
      for (int i1 = 0; i1 < n; ++i1) {
        const size_t r = (size_t)i1 + (size_t)n * (i2 + (size_t)n * i3);
        const double s = (double)((73 * i1 + 151 * i2 + 37 * i3 + 11) % 97) / 96.0;
        eps[r] = 1.0 + 12.0 * s;
        gam[r] = 0.2 * s;
      }
  if ((rc = check(fame_plan_create_field(&plan, n, 1, theta, lattice, eps, gam), NULL, "fame_plan_create_field")))
    goto out;
  if (cudaMalloc(&ev, sizeof(double) * 2 * len * k) != cudaSuccess ||
      cudaMalloc((void**)&g_dev, sizeof(double) * 2 * nq) != cudaSuccess) {
    fprintf(stderr, "cudaMalloc failed\n");
    rc = 1;
    goto out;
  }
  if ((rc = check(fame_lanczos(plan, FAME_C128, 0, k, 1e-12, 10000, 2 * k, NULL, 1e-13, ew, ev, NULL, NULL), plan,
                  "fame_lanczos")))
    goto out;
  /* Lanczos.m orders lambda = 1/omega descending: omega ascending */
  for (int i = 0; i < k; ++i) {
    om[i] = 1.0 / ew[i];
    w[i] = i == 1 ? -1.0 : i == 2 ? 1.0 : 0.0;
  }
  if ((rc = check(fame_eig_gradient(plan, k, NULL, ev, om, w, g_dev, g_dev + nq, 0, NULL), plan,
                  "fame_eig_gradient")))
    goto out;
  if (cudaMemcpy(g_host, g_dev, sizeof(double) * 2 * nq, cudaMemcpyDeviceToHost) != cudaSuccess) {
    fprintf(stderr, "cudaMemcpy failed\n");
    rc = 1;
    goto out;
  }
  for (int i = 0; i < k; ++i) printf("%.17g\n", om[i]);
  for (size_t r = 0; r < nq; ++r) printf("g %.17g %.17g\n", g_host[r], g_host[nq + r]);
out:
  if (plan) fame_plan_destroy(plan);
  if (ev) cudaFree(ev);
  if (g_dev) cudaFree(g_dev);
  free(eps);
  free(gam);
  free(g_host);
  free(ew);
  free(om);
  free(w);
  return rc;
}

int main(int argc, char** argv) {
  if (argc > 1 && !strcmp(argv[1], "grad"))
    return run_grad(argc > 2 ? atoi(argv[2]) : 6, argc > 3 ? atoi(argv[3]) : 4);
  const int n = argc > 1 ? atoi(argv[1]) : 6;
  const int k = argc > 2 ? atoi(argv[2]) : 4;
  const double pi = 3.14159265358979323846;
  /* FCC primitive vectors as columns, a = 1 (Physical_settings_woodpile.m:7) */
  const double lattice[9] = {0.0, 0.5, 0.5, 0.5, 0.0, 0.5, 0.5, 0.5, 0.0};
  const double theta[3] = {pi, 0.0, pi};
  const double wood[2] = {0.25, 1.0};
  const size_t nq = (size_t)n * n * n;
  unsigned char* phase = malloc(nq);
  double c6[72], tensors[2 * 54];
  double* ew = malloc(sizeof(double) * k);
  double* res = malloc(sizeof(double) * k);
  long long stats[4];
  fame_plan_t plan = NULL;
  int rc = 0;
  if (!phase || !ew || !res) return 1;

  if ((rc = check(fame_rasterize(n, lattice, FAME_SHAPE_WOODPILE, wood, 1, phase, FAME_HOST_PTR), NULL,
                  "fame_rasterize")))
    return rc;
  bi_isotropic(1.0, 0.0, c6);
  if ((rc = check(fame_material_blocks(c6, lattice, tensors), NULL, "fame_material_blocks"))) return rc;
  bi_isotropic(13.0, 0.2, c6);
  if ((rc = check(fame_material_blocks(c6, lattice, tensors + 54), NULL, "fame_material_blocks"))) return rc;
  if ((rc = check(fame_plan_create(&plan, n, 1, theta, phase, 2, tensors), NULL, "fame_plan_create"))) return rc;
  rc = check(fame_lanczos(plan, FAME_C128, 0, k, 1e-10, 10000, 2 * k, NULL, 1e-12, ew, NULL, res, stats), plan,
             "fame_lanczos");
  if (rc == FAME_OK) {
    double rmax = 0.0;
    for (int i = 0; i < k; ++i) {
      printf("%.17g\n", ew[i]);
      if (res[i] > rmax) rmax = res[i];
    }
    printf("res %.3e steps %lld\n", rmax, stats[0]);
  }
  fame_plan_destroy(plan);
  free(phase);
  free(ew);
  free(res);
  return rc;
}
