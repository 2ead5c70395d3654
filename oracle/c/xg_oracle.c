/*
 * C restatement of the two benchmark programs, loop for loop like the C that
 * the reference generates for them (xgrid/lang/generator.py:285-364): one
 * OpenMP full-grid loop nest per grid assignment, each cell filtered by its
 * mask value, implicit (in-place) sweeps through a scratch array, same
 * expression trees and evaluation order as the DSL source.  TEST
 * INFRASTRUCTURE: the oracle and the CPU baseline, never the product.
 *
 * Grids are row-major n x n (cell (i, j) at i*n + j; offset [di, dj] moves i by
 * di and j by dj).  Level 0 is written, level 1 is the previous step.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define AT(a, i, j) (a)[(int64_t)(i) * n + (j)]

/* u[0,0] = u[0,0] + c*(u[1,0] + u[-1,0] + u[0,1] + u[0,-1] - 4.0*u[0,0]); mask 1: u = 0.0 */
void xo_diffusion_step(double* u0, const double* u1, const int32_t* mask, int n, double c) {
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mask, i, j) == 0)
        AT(u0, i, j) = AT(u1, i, j) + c * ((((AT(u1, i + 1, j) + AT(u1, i - 1, j)) + AT(u1, i, j + 1)) +
                                           AT(u1, i, j - 1)) - 4.0 * AT(u1, i, j));
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mask, i, j) == 1) AT(u0, i, j) = 0.0;
}

typedef struct {
  double rho, nu, dt, dx, dy;
} xo_cavity_config;

static void pressure_boundaries(double* p0, const int32_t* mp, int n) {
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mp, i, j) == 1) AT(p0, i, j) = AT(p0, i, j - 1);
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mp, i, j) == 2) AT(p0, i, j) = AT(p0, i + 1, j);
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mp, i, j) == 3) AT(p0, i, j) = AT(p0, i, j + 1);
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mp, i, j) == 4) AT(p0, i, j) = 0.0;
}

/* The pressure update of the cavity program, reading `src` (neighbours) and b. */
static inline double pressure(const double* src, const double* b0, int n, int i, int j, xo_cavity_config g) {
  const double dx2 = g.dx * g.dx, dy2 = g.dy * g.dy;
  return ((((AT(src, i, j + 1) + AT(src, i, j - 1)) * dy2) + ((AT(src, i + 1, j) + AT(src, i - 1, j)) * dx2)) /
          (2.0 * (dx2 + dy2))) -
         (((dx2 * dy2) / (2.0 * (dx2 + dy2))) * AT(b0, i, j));
}

/* One call of the lid-driven cavity kernel: b from u, v; 1 + 50 Jacobi sweeps of
 * p with its four boundary masks after each; u, v momentum; velocity walls.
 * `scratch` holds n*n doubles. */
void xo_cavity_step(double* b0, double* p0, const double* p1, double* u0, const double* u1, double* v0,
                    const double* v1, const int32_t* mb, const int32_t* mp, const int32_t* mu, const int32_t* mv,
                    int n, xo_cavity_config g, double* scratch) {
  (void)mb;
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mb, i, j) == 0) {
        const double dudx = (AT(u1, i, j + 1) - AT(u1, i, j - 1)) / (2.0 * g.dx);
        const double dvdy = (AT(v1, i + 1, j) - AT(v1, i - 1, j)) / (2.0 * g.dy);
        const double dudy = (AT(u1, i + 1, j) - AT(u1, i - 1, j)) / (2.0 * g.dy);
        const double dvdx_num = (AT(v1, i, j + 1) - AT(v1, i, j - 1));
        const double t1 = (1.0 / g.dt) * (dudx + dvdy);
        const double t2 = dudx * dudx;
        const double t3 = 2.0 * ((dudy * dvdx_num) / (2.0 * g.dx));
        const double t4 = dvdy * dvdy;
        AT(b0, i, j) = g.rho * (((t1 - t2) - t3) - t4);
      }
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mp, i, j) == 0) AT(p0, i, j) = pressure(p1, b0, n, i, j, g);
  pressure_boundaries(p0, mp, n);
  for (int it = 0; it < 50; it++) {
#pragma omp parallel for collapse(2)
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        if (AT(mp, i, j) == 0) AT(scratch, i, j) = pressure(p0, b0, n, i, j, g);
#pragma omp parallel for collapse(2)
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        if (AT(mp, i, j) == 0) AT(p0, i, j) = AT(scratch, i, j);
    pressure_boundaries(p0, mp, n);
  }
  const double dx2 = g.dx * g.dx, dy2 = g.dy * g.dy;
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mu, i, j) == 0) {
        const double uc = AT(u1, i, j), vc = AT(v1, i, j);
        AT(u0, i, j) = (((uc - (((uc * g.dt) / g.dx) * (uc - AT(u1, i, j - 1)))) -
                         (((vc * g.dt) / g.dy) * (uc - AT(u1, i - 1, j)))) -
                        ((g.dt / ((2.0 * g.rho) * g.dx)) * (AT(p0, i, j + 1) - AT(p0, i, j - 1)))) +
                       (g.nu * (((g.dt / dx2) * ((AT(u1, i, j + 1) - (2.0 * uc)) + AT(u1, i, j - 1))) +
                                ((g.dt / dy2) * ((AT(u1, i + 1, j) - (2.0 * uc)) + AT(u1, i - 1, j)))));
      }
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mv, i, j) == 0) {
        const double uc = AT(u1, i, j), vc = AT(v1, i, j);
        AT(v0, i, j) = (((vc - (((uc * g.dt) / g.dx) * (vc - AT(v1, i, j - 1)))) -
                         (((vc * g.dt) / g.dy) * (vc - AT(v1, i - 1, j)))) -
                        ((g.dt / ((2.0 * g.rho) * g.dy)) * (AT(p0, i + 1, j) - AT(p0, i - 1, j)))) +
                       (g.nu * (((g.dt / dx2) * ((AT(v1, i, j + 1) - (2.0 * vc)) + AT(v1, i, j - 1))) +
                                ((g.dt / dy2) * ((AT(v1, i + 1, j) - (2.0 * vc)) + AT(v1, i - 1, j)))));
      }
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mu, i, j) == 1) AT(u0, i, j) = 0.0;
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mv, i, j) == 1) AT(v0, i, j) = 0.0;
#pragma omp parallel for collapse(2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (AT(mu, i, j) == 2) AT(u0, i, j) = 1.0;
}
