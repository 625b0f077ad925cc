/* abi_check.c -- the C-ABI from plain C (no GPU needed): headers compile as
   C99, the library links, host-only entry points answer, errors report. */
#include <stdio.h>
#include <string.h>
#include "gbvol.h"
#include "barney_gb300.h"

int main(void) {
  int dims[3] = {100, 60, 33}, mc[3] = {0, 0, 0};
  size_t vb = 0, sb = 0;
  int shape[3] = {4, 3, 2};
  int n = 0, lower[2 * 16];
  int k;
  if (gbv_mc_dims(dims, 8, mc) != GBV_OK) return 1;
  printf("mc_dims %d %d %d\n", mc[0], mc[1], mc[2]);
  if (gbv_brick_store_bytes_shaped(dims, GBV_VOXEL_U8_SCALED, shape, &vb, &sb) != GBV_OK) return 2;
  printf("store_bytes %zu %zu\n", vb, sb);
  if (gbv_tile_partition(100, 70, 1, 3, &n, lower) != GBV_OK) return 3;
  printf("tiles %d", n);
  for (k = 0; k < n; k++) printf(" %d,%d", lower[2 * k], lower[2 * k + 1]);
  printf("\n");
  printf("tile_bytes %zu\n", gbv_compressed_tile_bytes());
  if (gbv_mc_dims(dims, 0, mc) != GBV_ERROR_INVALID_ARGUMENT) return 4;
  printf("error \"%s\"\n", gbv_last_error());
  printf("version %d\n", gbv_version());
  return 0;
}
