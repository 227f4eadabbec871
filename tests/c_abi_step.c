/* A plain-C caller of the engine's C ABI (include/flowlab_gb300.h), the way
 * a Node addon or any non-Python host binds it: a 64 x 64 closed box with a
 * warm blob of dye, one fl_step_host call (upload, step, read back), then
 * the velocity's largest magnitude. Exit status: 0 after a step, 2 when
 * fl_create reports that no CUDA device is usable (FL_EDEVICE, with
 * fl_last_error(NULL) printed), 1 on any other failure. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "flowlab_gb300.h"

int main(void) {
  const int nx = 64, ny = 64;
  fl_params prm;
  fl_default_params(&prm);
  prm.scheme = FL_MACCORMACK;
  prm.beta = 1.0;
  fl_engine* e = NULL;
  int st = fl_create(nx, ny, 1.0 / nx, 1, &prm, 0, &e);
  if (st == FL_EDEVICE) {
    printf("no device: %s\n", fl_last_error(NULL));
    return 2;
  }
  if (st != FL_OK) {
    printf("create failed (%d): %s\n", st, fl_last_error(NULL));
    return 1;
  }
  const long nu = (long)(nx + 1) * ny, nv = (long)nx * (ny + 1), nc = (long)nx * ny;
  float* u = calloc(nu, sizeof(float));
  float* v = calloc(nv, sizeof(float));
  float* p = calloc(nc, sizeof(float));
  float* dye = calloc(3 * nc, sizeof(float));
  uint8_t* label = calloc(nc, 1); /* all Fluid: a closed box */
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      const double x = (i + 0.5) / nx - 0.5, y = (j + 0.5) / ny - 0.25;
      dye[i + (long)j * nx] = (float)exp(-(x * x + y * y) / 0.01); /* channel 0: temperature */
    }
  int cycles = 0;
  st = fl_step_host(e, FL_F32, u, v, p, label, dye, u, v, p, dye, &cycles);
  if (st != FL_OK) {
    printf("step failed (%d): %s\n", st, fl_last_error(e));
    fl_destroy(e);
    return 1;
  }
  float vmax = 0.0f;
  for (long k = 0; k < nv; k++) vmax = fabsf(v[k]) > vmax ? fabsf(v[k]) : vmax;
  printf("stepped: %d V-cycles, max |v| %g\n", cycles, vmax);
  fl_destroy(e);
  free(u);
  free(v);
  free(p);
  free(dye);
  free(label);
  return 0;
}
