/* Sanitizer driver for the CPU oracle — TEST INFRASTRUCTURE ONLY.
 *
 * Built by `make -C oracle sanitize` with AddressSanitizer and UndefinedBehaviorSanitizer
 * (every UB report is fatal) and run by the CPU test suite. It walks every entry point of
 * sts_oracle.c over tiny and ragged grids (8x8, 17x9, 5x12, periodic 12x10 with inhomogeneous
 * faces), both LSRK methods, FP64 and mixed stages, every controller, the SSP methods, the
 * power iteration, the Krylov solvers and the multigrid cycle, and states holding NaN and Inf,
 * so out-of-bounds accesses, leaks, overflowing integer conversions and other undefined
 * behaviour in the oracle surface here instead of as silent parity drift. Prints one line per
 * group and "sanitize_check: ok" at the end.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sts_oracle.h"

static double* vec(long n) { return (double*)calloc((size_t)n, sizeof(double)); }

static void fill(double* v, long n, unsigned seed)
{
  unsigned s = seed * 2654435761u + 1u;
  for (long i = 0; i < n; ++i)
  {
    s    = s * 1664525u + 1013904223u;
    v[i] = (double)(s >> 8) / 16777216.0 - 0.5;
  }
}

static orc_opts opts(int method, int mixed, int controller)
{
  orc_opts o;
  memset(&o, 0, sizeof(o));
  o.method       = method;
  o.mixed        = mixed;
  o.controller   = controller;
  o.smax         = 200;
  o.dee_maxiters = 100;
  o.dom_eig_freq = 25;
  o.maxsteps     = 0;
  o.rtol         = 1e-6;
  o.atol         = 1e-10;
  o.eig_safety   = 1.01;
  o.dee_reltol   = 0.01;
  return o;
}

static int evolve(orc_prob* p, const orc_opts* o, double tout, const double* y0, long* nst)
{
  long n = (long)p->nx * p->ny;
  double* y = vec(n);
  memcpy(y, y0, n * sizeof(double));
  orc_state st;
  orc_state_init(&st, 0.0);
  int rc = orc_lsrk_evolve(p, o, &st, tout * 0.5, y);
  if (rc == 0) rc = orc_lsrk_evolve(p, o, &st, tout, y);
  *nst = st.nst;
  orc_state_free(&st);
  free(y);
  return rc;
}

int main(void)
{
  const int grids[][3] = {{0, 8, 8}, {0, 17, 9}, {1, 5, 12}, {2, 12, 10}};
  int fails = 0;
  for (int g = 0; g < 4; ++g)
  {
    const int kind = grids[g][0], nx = grids[g][1], ny = grids[g][2];
    orc_prob* p = orc_prob_create(kind, nx, ny, 1.0, 0.3, kind == 2, -M_PI, M_PI, -6.0, 6.0);
    const long n = (long)nx * ny;
    double *y0 = vec(n), *f = vec(n), *w = vec(n), *z = vec(n), *b = vec(n), *x = vec(n);
    orc_initial(p, y0);
    orc_rhs(p, 0.0, y0, f);
    orc_rhs_ref(p, 0.0, y0, f);
    orc_apply_A(p, y0, w);
    (void)orc_dom_eig(p);
    memcpy(z, y0, n * sizeof(double));
    double lam = 0.0;
    (void)orc_power_iteration(p, z, 100, 0.01, &lam);
    (void)orc_xsum(y0, n);
    (void)orc_xdot(y0, f, n);
    for (long i = 0; i < n; ++i) w[i] = 1.0 / (1e-6 * fabs(y0[i]) + 1e-10);
    (void)orc_wrms(f, w, n);
    (void)orc_maxnorm(f, n);
    if (kind == 0) orc_exact(p, 0.1, z);

    long nst = 0;
    for (int method = 0; method < 2; ++method)
      for (int mixed = 0; mixed < (kind == 2 ? 1 : 2); ++mixed)
        for (int controller = 0; controller < 6; ++controller)
        {
          orc_opts o = opts(method, mixed, controller);
          o.internaleig = (controller == 1);
          if (evolve(p, &o, 0.01, y0, &nst) != 0) ++fails;
        }
    {
      /* stage cap and fixed step */
      orc_opts o = opts(1, 0, 0);
      o.smax = 3;
      if (evolve(p, &o, 0.01, y0, &nst) != 0) ++fails;
      o        = opts(0, 0, 0);
      o.hfixed = 1e-4;
      if (evolve(p, &o, 0.001, y0, &nst) != 0) ++fails;
    }
    const long nst_fixed = nst;
    if (kind != 2)
    {
      const int ssp[][2] = {{2, 4}, {3, 9}, {4, 10}};
      for (int k = 0; k < 3; ++k)
      {
        orc_opts o = opts(0, 0, 0);
        orc_state st;
        orc_state_init(&st, 0.0);
        memcpy(z, y0, n * sizeof(double));
        if (orc_ssp_evolve(p, &o, ssp[k][0], ssp[k][1], &st, 0.002, z) != 0) ++fails;
        orc_state_free(&st);
      }
    }
    /* non-finite states fail cleanly */
    for (int k = 0; k < 3; ++k)
    {
      memcpy(z, y0, n * sizeof(double));
      z[n / 2] = (k == 0) ? NAN : (k == 1 ? INFINITY : -INFINITY);
      orc_opts o = opts(k & 1, k == 2 && kind != 2, 0);
      if (evolve(p, &o, 0.01, z, &nst) != -3) ++fails;
    }
    /* Krylov solvers and the multigrid cycle on (I - gamma A) x = b */
    if (kind != 2)
    {
      fill(b, n, (unsigned)g + 1u);
      const double gamma = 1e-3;
      double rel = 0.0;
      int it = 0, nl = 0;
      (void)orc_pcg(p, gamma, 1, b, x, 1e-10, 1000, &rel);
      (void)orc_pcg_generic(p, gamma, 1, b, x, 1e-10, 1000, &it, &rel);
      for (int gs = 0; gs < 2; ++gs)
      {
        (void)orc_spgmr(p, gamma, 1, b, x, 1e-10, 5, 20, gs, &it, &rel);
        (void)orc_spfgmr(p, gamma, 1, b, x, 1e-10, 5, 20, gs, &it, &rel);
      }
      for (int relax = 1; relax <= 2; ++relax)
      {
        (void)orc_pfmg_vcycle(p, gamma, relax, 2, b, z, &nl);
        (void)orc_pcg_pfmg(p, gamma, relax, 2, b, x, 1e-10, 200, &it, &rel);
      }
      long its = 0;
      memcpy(z, y0, n * sizeof(double));
      (void)orc_sdirk2(p, 0.0, 1e-4, 2, 1e-10, 1000, z, &its);
      (void)orc_sdirk2_ls(p, 0.0, 1e-4, 2, 1e-10, 1, 10, 5, 1, 1, z, &its);
      (void)orc_sdirk2_pfmg(p, 0.0, 1e-4, 2, 1e-10, 200, 2, 2, z, &its);
    }
    printf("grid kind %d %dx%d: ok (%ld fixed steps)\n", kind, nx, ny, nst_fixed);
    if (nst_fixed != 10) ++fails;
    free(y0);
    free(f);
    free(w);
    free(z);
    free(b);
    free(x);
    orc_prob_free(p);
  }
  /* step rules at the edges of their domains */
  double hm;
  for (int method = 0; method < 2; ++method)
  {
    if (orc_stages_needed(method, NAN, 1e4, 200, &hm) != 2) ++fails;
    if (orc_stages_needed(method, 1e300, 1e300, 200, &hm) != 1000000000) ++fails;
    (void)orc_stages_needed(method, 1e-3, 0.0, 200, &hm);
  }
  for (int c = 0; c < 6; ++c)
  {
    (void)orc_controller(c, 1e-3, 0.0, 0.0, 0.0, 0.0, 0);
    (void)orc_controller(c, 1e-3, NAN, 1.0, 1.0, 1e-3, 3);
  }
  (void)orc_pow(0.0, 0.5);
  (void)orc_pow(1e-300, -0.25);
  for (int s = 2; s <= 200; s += 37)
  {
    double mu[201], nu[201], mus[201], aj[201], cj[201];
    (void)orc_stage_coeffs(0, s, mu, nu, mus, aj, cj);
    (void)orc_stage_coeffs(1, s, mu, nu, mus, aj, cj);
  }
  if (fails)
  {
    printf("sanitize_check: %d unexpected return codes\n", fails);
    return 1;
  }
  printf("sanitize_check: ok\n");
  return 0;
}
