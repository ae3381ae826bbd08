/* Oracle, plain C (test infrastructure only: the tests and the CPU baseline of bench.py load
   it; nothing in autopdex_gb300/ links or calls it).

   A second, independent float64 restatement of two pieces of the reference's path, written
   in closed form where oracle/elements.py differentiates with torch.func:

   * orc_neo_hooke_hex8: the Galerkin neo-Hooke element of
     models.isoparametric_domain_element_galerkin + hyperelastic_steady_state_weak +
     neo_hooke (models.py:1616-1718, :917-1000, :1122-1146) on the 8-node brick of
     fem_iso_line_quad_brick (spaces.py:12057-12081, physical gradients :12162-12190) with the
     2 x 2 x 2 Gauss rule of seeder.gauss_legendre_nd(3, 2) (seeder.py:382-386, :1046-1062).
     psi = mu/2 (tr C - 3 - 2 ln J) + lam/4 (J^2 - 1 - 2 ln J) gives
       P = mu F + c F^-T,  c = lam/2 (J^2 - 1) - mu,
       dP_iJ/dF_kL = mu d_ik d_JL + lam J^2 F^-T_iJ F^-T_kL - c F^-T_iL F^-T_kJ,
     so with g_a = dN_a/dX and h_a = F^-T g_a per Gauss point (weight w, det J):
       R_ai  += w det J (mu (F g_a)_i + c h_ai)
       K_aibk += w det J (mu (g_a . g_b) d_ik + lam J^2 h_ai h_bk - c h_ak h_bi).
     The Jacobian's determinant keeps its sign (models.py:1249-1254 multiply by the signed
     matrix_det), as the reference does.
   * orc_pcg_csr: Jacobi-preconditioned CG on a float64 CSR matrix (the algorithm of
     linear_solve_jax's 'cg' + 'jacobi', solver.py:1084-1116), a fixed number of iterations,
     OpenMP-parallel products, updates and dots.

   Built by oracle/build_oracle.py with gcc -O3 -fopenmp. */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* threads the parallel loops use (1 when built without OpenMP) */
int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static void inv3(const double m[3][3], double r[3][3], double* det) {
  const double d = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                   m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                   m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  const double s = 1.0 / d;
  r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * s;
  r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * s;
  r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * s;
  r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * s;
  r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * s;
  r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * s;
  r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * s;
  r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * s;
  r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * s;
  *det = d;
}

/* one element: xI, uI (8 x 3, node order of the 8-node brick) -> R (24), K (24 x 24) */
static void neo_hooke_hex8(const double* xI, const double* uI, double lam, double mu, double* R, double* K) {
  static const int sgn[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const double gp[2] = {2.0 * 0.21132486540518713 - 1.0, 2.0 * 0.7886751345948129 - 1.0};
  memset(R, 0, 24 * sizeof(double));
  if (K) memset(K, 0, 576 * sizeof(double));
  for (int q = 0; q < 8; ++q) {
    const double xi[3] = {gp[q & 1], gp[(q >> 1) & 1], gp[(q >> 2) & 1]};  /* first coordinate fastest */
    double dN[8][3];
    for (int a = 0; a < 8; ++a) {
      double f[3];
      for (int d = 0; d < 3; ++d) f[d] = 0.5 * (1.0 + sgn[a][d] * xi[d]);
      dN[a][0] = 0.5 * sgn[a][0] * f[1] * f[2];
      dN[a][1] = 0.5 * sgn[a][1] * f[0] * f[2];
      dN[a][2] = 0.5 * sgn[a][2] * f[0] * f[1];
    }
    double J[3][3] = {{0}}, Ji[3][3], detJ;
    for (int a = 0; a < 8; ++a)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) J[i][j] += xI[3 * a + i] * dN[a][j];
    inv3(J, Ji, &detJ);
    double g[8][3];
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d) g[a][d] = dN[a][0] * Ji[0][d] + dN[a][1] * Ji[1][d] + dN[a][2] * Ji[2][d];
    double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, Fi[3][3], JF;
    for (int a = 0; a < 8; ++a)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) F[i][j] += uI[3 * a + i] * g[a][j];
    inv3(F, Fi, &JF);
    const double c = 0.5 * lam * (JF * JF - 1.0) - mu, lj2 = lam * JF * JF;
    const double wd = detJ; /* Gauss weights 1 */
    double h[8][3];
    for (int a = 0; a < 8; ++a)
      for (int i = 0; i < 3; ++i) h[a][i] = Fi[0][i] * g[a][0] + Fi[1][i] * g[a][1] + Fi[2][i] * g[a][2];
    for (int a = 0; a < 8; ++a)
      for (int i = 0; i < 3; ++i) {
        const double Fg = F[i][0] * g[a][0] + F[i][1] * g[a][1] + F[i][2] * g[a][2];
        R[3 * a + i] += wd * (mu * Fg + c * h[a][i]);
      }
    if (!K) continue;
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b) {
        const double gg = g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2];
        for (int i = 0; i < 3; ++i)
          for (int k = 0; k < 3; ++k)
            K[(3 * a + i) * 24 + 3 * b + k] +=
                wd * ((i == k ? mu * gg : 0.0) + lj2 * h[a][i] * h[b][k] - c * h[a][k] * h[b][i]);
      }
  }
}

/* all elements: conn (n_e x 8), coords and dofs (n_nodes x 3) -> R_e (n_e x 24) and, unless
   K_e is NULL, K_e (n_e x 576); E, nu -> Lame parameters as models.py:955-956 */
void orc_neo_hooke_hex8(int64_t n_e, const int64_t* conn, const double* coords, const double* dofs, double E,
                        double nu, double* R_e, double* K_e) {
  const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = E / (2.0 * (1.0 + nu));
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < n_e; ++e) {
    double xI[24], uI[24];
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d) {
        xI[3 * a + d] = coords[3 * conn[8 * e + a] + d];
        uI[3 * a + d] = dofs[3 * conn[8 * e + a] + d];
      }
    neo_hooke_hex8(xI, uI, lam, mu, R_e + 24 * e, K_e ? K_e + 576 * e : 0);
  }
}

/* Jacobi-PCG on CSR (rowptr n+1, col nnz, val nnz) for `iters` iterations from x = 0, with
   caller-provided work vectors (n each, dinv included); returns (r, r) at the end */
double orc_pcg_csr(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, const double* b,
                   double* x, double* r, double* z, double* p, double* q, double* dinv, int iters) {
  double rz = 0.0;
#pragma omp parallel for reduction(+ : rz)
  for (int64_t i = 0; i < n; ++i) {
    double d = 0.0;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (col[k] == i) d = val[k];
    dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
    x[i] = 0.0;
    r[i] = b[i];
    z[i] = dinv[i] * b[i];
    p[i] = z[i];
    rz += r[i] * z[i];
  }
  double rr = 0.0;
  for (int it = 0; it < iters; ++it) {
    double pq = 0.0;
#pragma omp parallel for reduction(+ : pq)
    for (int64_t i = 0; i < n; ++i) {
      double s = 0.0;
      for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) s += val[k] * p[col[k]];
      q[i] = s;
      pq += p[i] * s;
    }
    const double alpha = rz / pq;
    double rz_new = 0.0;
    rr = 0.0;
#pragma omp parallel for reduction(+ : rz_new, rr)
    for (int64_t i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = dinv[i] * r[i];
      rz_new += r[i] * z[i];
      rr += r[i] * r[i];
    }
    const double beta = rz_new / rz;
    rz = rz_new;
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  return rr;
}
