/* A plain C99 consumer of the sweep library's C ABI (include/subsweep_gpu.h): what a
 * Rust or C caller links against.  Built and run by tests/test_abi_consumer.py.
 *
 * It reads the default parameters and a direction table, then creates a handle for a
 * 4-cell column along x (LOCAL faces between neighbours, BOUNDARY faces elsewhere) and,
 * when a device is present, runs two steps and reads the fields back.  Prints one line:
 *   "create <status> <message>" and, after a successful create, "fields <x0> <T0>". */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "subsweep_gpu.h"

#define N 4

int main(void) {
  sw_params p;
  double dirs[3 * 84];
  int64_t row_ptr[N + 1];
  int32_t nbr[6 * N];
  uint8_t kind[6 * N];
  double area[6 * N], normal[18 * N], volume[N], size[N];
  double density[N], xhii[N], temperature[N], source[N];
  static const double axes[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  sw_grid_csr grid;
  sw_cell_init init;
  sw_handle* h = NULL;
  sw_status st;
  int c, f, d, e = 0;

  if (sw_default_params(&p) != SW_OK || p.num_directions != 84 || p.num_timestep_levels != 1) return 10;
  if (sw_directions_from_num(84, dirs) != SW_OK) return 11;
  for (d = 0; d < 84; ++d) {
    const double n2 = dirs[3 * d] * dirs[3 * d] + dirs[3 * d + 1] * dirs[3 * d + 1] + dirs[3 * d + 2] * dirs[3 * d + 2];
    if (fabs(n2 - 1.0) > 1e-5) return 12; /* the reference's tables are literals to ~1e-7 */
  }
  if (sw_directions_from_num(7, dirs) != SW_ERR_INVALID_ARG) return 13;

  for (c = 0; c < N; ++c) {
    row_ptr[c] = e;
    for (f = 0; f < 6; ++f, ++e) {
      const int interior = (f == 0 && c + 1 < N) || (f == 1 && c > 0);
      nbr[e] = interior ? (f == 0 ? c + 1 : c - 1) : -1;
      kind[e] = (uint8_t)(interior ? SW_FACE_LOCAL : SW_FACE_BOUNDARY);
      area[e] = 1e32;
      memcpy(&normal[3 * e], axes[f], sizeof axes[f]);
    }
    volume[c] = 1e48;
    size[c] = 1e16;
    density[c] = 1e-24;
    xhii[c] = 1e-10;
    temperature[c] = 1e4;
    source[c] = c == 0 ? 1e49 : 0.0;
  }
  row_ptr[N] = e;

  p.num_directions = 16;
  p.periodic = 0;
  p.max_timestep = 3.15576e13;
  p.precision = SW_PRECISION_MIXED;
  grid.num_cells = N;
  grid.row_ptr = row_ptr;
  grid.nbr = nbr;
  grid.kind = kind;
  grid.area = area;
  grid.normal = normal;
  grid.volume = volume;
  grid.size = size;
  init.density = density;
  init.ionized_hydrogen_fraction = xhii;
  init.temperature = temperature;
  init.source = source;

  st = sw_create(&p, &grid, &init, &h);
  printf("create %d %s\n", (int)st, st == SW_OK ? "" : sw_last_error(NULL));
  if (st != SW_OK) return 0;
  {
    double elapsed, x[N], t[N], dt[N], rate[N];
    if (sw_step(h, &elapsed) != SW_OK || sw_step(h, &elapsed) != SW_OK) return 20;
    if (sw_get_fields(h, x, t, dt, rate) != SW_OK) return 21;
    printf("fields %.17g %.17g\n", x[0], t[0]);
  }
  sw_destroy(h);
  return 0;
}
