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

/* Jacobi-PCG on CSR (rowptr n+1, col nnz, val nnz) from x = 0, with caller-provided work
   vectors (n each, dinv included): at most `iters` iterations, fewer once (r, r) <= rtol^2 (b, b)
   (rtol = 0: exactly `iters`); returns (r, r) at the end and the iteration count in *done */
double orc_pcg_csr_tol(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, const double* b,
                       double* x, double* r, double* z, double* p, double* q, double* dinv, int iters, double rtol,
                       int* done) {
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
  double bb = 0.0;
#pragma omp parallel for reduction(+ : bb)
  for (int64_t i = 0; i < n; ++i) bb += b[i] * b[i];
  const double stop = rtol * rtol * bb;
  double rr = bb;
  int it = 0;
  for (; it < iters && !(rtol > 0.0 && rr <= stop); ++it) {
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
  if (done) *done = it;
  return rr;
}

/* exactly `iters` iterations (the fixed-count form) */
double orc_pcg_csr(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, const double* b,
                   double* x, double* r, double* z, double* p, double* q, double* dinv, int iters) {
  return orc_pcg_csr_tol(n, rowptr, col, val, b, x, r, z, p, q, dinv, iters, 0.0, 0);
}

/* ---- Q1 quads and bricks, 2-node boundary lines, in closed form ------------------------

   orc_q1_elements: element residuals and tangents of the models of the backend's descriptors
   on Q1 quads (dim 2, nodes (-1,-1) (1,-1) (1,1) (-1,1): spaces.py:1913-1922) and Q1 bricks
   (dim 3: spaces.py:12057-12081), 2 x 2 (x 2) Gauss-Legendre points with unit weights, the
   first coordinate fastest (seeder.py:382-386, :1046-1062), physical gradients g = dN/dxi J^-1
   (spaces.py:12162-12190), signed det J (models.py:1249-1254):
     model 0, Poisson user potential 1/2 |grad u|^2 - b u with
       b = amp (sin(freq x.x) - cos(freq |x - c|^2))  (tests/test_dicts_as_dofs_user_potential.py:25-35)
       params amp, freq, c_x, c_y:   R_a = sum w detJ (grad u . g_a - b N_a),  K_ab = sum w detJ g_a . g_b
     model 1, heat user potential 1/2 k_e |grad u|^2 - f u (models.py:1188-1269), params f,
       elem_field k_e:               R_a = sum w detJ (k_e grad u . g_a - f N_a), K_ab = sum w detJ k_e g_a . g_b
     model 2, Galerkin neo-Hooke (plane strain in 2-D, F33 = 1; models.py:917-1000, :1122-1146,
       :1616-1718), params E, nu:    R_ai = sum w detJ P_iJ g_aJ,
       K_aibk = sum w detJ (mu g_a.g_b d_ik + lam J^2 h_ai h_bk - c h_ak h_bi), h = F^-T g,
       c = lam/2 (J^2 - 1) - mu.  `accurate` = 0 forms J = det F and P = mu F + c F^-T as the
       reference's AD of psi does; `accurate` = 1 evaluates the same P from H = grad u as
       mu (H + I - F^-T) + lam/2 (J - 1)(J + 1) F^-T with J - 1 = tr H + i2(H) + det H and
       I - F^-T = (H^T + (i2 + det H) I - cof H) / J, free of the cancellation that lam turns
       into a stress error of lam eps when J ~ 1 (nearly incompressible materials).
     model 4, backward-Euler heat 'user residual' (models.py:1272-1357), params k0, k2, rho_c,
       dt, node_field T_n:  R_a = sum w detJ (rho_c (T - T_n)/dt N_a + (k0 + k2 T^2) grad T . g_a),
       K_ab = sum w detJ (rho_c/dt N_a N_b + k(T) g_a . g_b + 2 k2 T N_b grad T . g_a).
   Outputs R_e (n_e x m) and, unless K_e is NULL, K_e (n_e x m x m), m = nen ndof, DOFs
   node-major (dof = node ndof + component). */
static void q1_point(int dim, int q, const double* xI, double N[8], double g[8][3], double* wdet, double x[3]) {
  const double gp[2] = {-0.57735026918962584, 0.57735026918962584};
  static const int s2[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  static const int s3[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                               {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const int nen = dim == 2 ? 4 : 8;
  double xi[3] = {gp[q & 1], gp[(q >> 1) & 1], dim == 3 ? gp[(q >> 2) & 1] : 0.0};
  double dN[8][3];
  for (int a = 0; a < nen; ++a) {
    double f[3];
    for (int d = 0; d < dim; ++d) f[d] = 0.5 * (1.0 + (dim == 2 ? s2[a][d] : s3[a][d]) * xi[d]);
    if (dim == 2) {
      N[a] = f[0] * f[1];
      dN[a][0] = 0.5 * s2[a][0] * f[1];
      dN[a][1] = 0.5 * s2[a][1] * f[0];
    } else {
      N[a] = f[0] * f[1] * f[2];
      dN[a][0] = 0.5 * s3[a][0] * f[1] * f[2];
      dN[a][1] = 0.5 * s3[a][1] * f[0] * f[2];
      dN[a][2] = 0.5 * s3[a][2] * f[0] * f[1];
    }
  }
  double J[3][3] = {{0}}, Ji[3][3] = {{0}}, det;
  for (int a = 0; a < nen; ++a)
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) J[i][j] += xI[dim * a + i] * dN[a][j];
  if (dim == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
  } else {
    inv3(J, Ji, &det);
  }
  for (int a = 0; a < nen; ++a)
    for (int d = 0; d < dim; ++d) {
      double v = 0.0;
      for (int k = 0; k < dim; ++k) v += dN[a][k] * Ji[k][d];
      g[a][d] = v;
    }
  for (int d = 0; d < 3; ++d) x[d] = 0.0;
  for (int a = 0; a < nen; ++a)
    for (int d = 0; d < dim; ++d) x[d] += N[a] * xI[dim * a + d];
  *wdet = det; /* unit Gauss weights */
}

/* P, F^-1, J of the neo-Hooke law from H = grad u (3 x 3, plane strain with zero third row and
   column); accurate: the cancellation-free form described above */
static void neo_hooke_law(const double H[3][3], double lam, double mu, int accurate, double P[3][3],
                          double Fi[3][3], double* Jout) {
  double F[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
  double J;
  inv3(F, Fi, &J);
  if (!accurate) {
    const double c = 0.5 * lam * (J * J - 1.0) - mu;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) P[i][j] = mu * F[i][j] + c * Fi[j][i];
    *Jout = J;
    return;
  }
  const double i2 = (H[0][0] * H[1][1] - H[0][1] * H[1][0]) + (H[0][0] * H[2][2] - H[0][2] * H[2][0]) +
                    (H[1][1] * H[2][2] - H[1][2] * H[2][1]);
  const double dH = H[0][0] * (H[1][1] * H[2][2] - H[1][2] * H[2][1]) - H[0][1] * (H[1][0] * H[2][2] - H[1][2] * H[2][0]) +
                    H[0][2] * (H[1][0] * H[2][1] - H[1][1] * H[2][0]);
  const double jm1 = (H[0][0] + H[1][1] + H[2][2]) + (i2 + dH);
  J = 1.0 + jm1;
  double C[3][3], cofH[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const int i1 = (i + 1) % 3, i2_ = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      C[i][j] = F[i1][j1] * F[i2_][j2] - F[i1][j2] * F[i2_][j1];
      cofH[i][j] = H[i1][j1] * H[i2_][j2] - H[i1][j2] * H[i2_][j1];
    }
  const double pl = 0.5 * lam * jm1 * (2.0 + jm1);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      Fi[j][i] = C[i][j] / J;
      const double m = (H[j][i] + (i == j ? i2 + dH : 0.0) - cofH[i][j]) / J;
      P[i][j] = mu * (H[i][j] + m) + pl * C[i][j] / J;
    }
  *Jout = J;
}

static void q1_element(int model, int dim, const double* xI, const double* uI, const double* p, double kfield,
                       const double* TnI, int accurate, double* R, double* K) {
  const int nen = dim == 2 ? 4 : 8, nq = nen, ndof = model == 2 ? dim : 1, m = nen * ndof;
  memset(R, 0, sizeof(double) * m);
  if (K) memset(K, 0, sizeof(double) * m * m);
  for (int q = 0; q < nq; ++q) {
    double N[8], g[8][3], wd, x[3];
    q1_point(dim, q, xI, N, g, &wd, x);
    if (model == 2) {
      const double E = p[0], nu = p[1];
      const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = E / (2.0 * (1.0 + nu));
      double H[3][3] = {{0}}, P[3][3], Fi[3][3], J;
      for (int a = 0; a < nen; ++a)
        for (int i = 0; i < dim; ++i)
          for (int j = 0; j < dim; ++j) H[i][j] += uI[dim * a + i] * g[a][j];
      neo_hooke_law(H, lam, mu, accurate, P, Fi, &J);
      for (int a = 0; a < nen; ++a)
        for (int i = 0; i < dim; ++i) {
          double v = 0.0;
          for (int j = 0; j < dim; ++j) v += P[i][j] * g[a][j];
          R[dim * a + i] += wd * v;
        }
      if (!K) continue;
      const double c = 0.5 * lam * (J * J - 1.0) - mu, lj2 = lam * J * J;
      double h[8][3];
      for (int a = 0; a < nen; ++a)
        for (int i = 0; i < dim; ++i) {
          double v = 0.0;
          for (int j = 0; j < dim; ++j) v += Fi[j][i] * g[a][j];
          h[a][i] = v;
        }
      for (int a = 0; a < nen; ++a)
        for (int b = 0; b < nen; ++b) {
          double gg = 0.0;
          for (int d = 0; d < dim; ++d) gg += g[a][d] * g[b][d];
          for (int i = 0; i < dim; ++i)
            for (int k = 0; k < dim; ++k)
              K[(dim * a + i) * m + dim * b + k] +=
                  wd * ((i == k ? mu * gg : 0.0) + lj2 * h[a][i] * h[b][k] - c * h[a][k] * h[b][i]);
        }
      continue;
    }
    double u = 0.0, gu[3] = {0, 0, 0};
    for (int a = 0; a < nen; ++a) {
      u += N[a] * uI[a];
      for (int d = 0; d < dim; ++d) gu[d] += uI[a] * g[a][d];
    }
    double kq = 1.0, src = 0.0, mass = 0.0, dk = 0.0, Tn = 0.0;
    if (model == 0) {
      double r1 = 0.0, r2 = 0.0;
      for (int d = 0; d < dim; ++d) {
        r1 += x[d] * x[d];
        r2 += (x[d] - p[2 + d]) * (x[d] - p[2 + d]);
      }
      src = p[0] * (sin(p[1] * r1) - cos(p[1] * r2));
    } else if (model == 1) {
      kq = kfield;
      src = p[0];
    } else { /* model 4 */
      for (int a = 0; a < nen; ++a) Tn += N[a] * TnI[a];
      kq = p[0] + p[1] * u * u;
      dk = 2.0 * p[1] * u;
      mass = p[2] / p[3];
      src = -mass * (u - Tn);
    }
    for (int a = 0; a < nen; ++a) {
      double gg = 0.0;
      for (int d = 0; d < dim; ++d) gg += gu[d] * g[a][d];
      R[a] += wd * (kq * gg - src * N[a]);
    }
    if (!K) continue;
    for (int a = 0; a < nen; ++a) {
      double gua = 0.0;
      for (int d = 0; d < dim; ++d) gua += gu[d] * g[a][d];
      for (int b = 0; b < nen; ++b) {
        double gg = 0.0;
        for (int d = 0; d < dim; ++d) gg += g[a][d] * g[b][d];
        double v = kq * gg;
        if (model == 4) v += mass * N[a] * N[b] + dk * N[b] * gua;
        K[a * m + b] += wd * v;
      }
    }
  }
}

void orc_q1_elements(int model, int dim, int64_t n_e, const int64_t* conn, const double* coords,
                     const double* dofs, const double* params, const double* elem_field,
                     const double* node_field, int accurate, double* R_e, double* K_e) {
  const int nen = dim == 2 ? 4 : 8, ndof = model == 2 ? dim : 1, m = nen * ndof;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < n_e; ++e) {
    double xI[24], uI[24], TnI[8];
    for (int a = 0; a < nen; ++a) {
      const int64_t nd = conn[nen * e + a];
      for (int d = 0; d < dim; ++d) xI[dim * a + d] = coords[dim * nd + d];
      for (int c = 0; c < ndof; ++c) uI[ndof * a + c] = dofs[ndof * nd + c];
      TnI[a] = node_field ? node_field[nd] : 0.0;
    }
    q1_element(model, dim, xI, uI, params, elem_field ? elem_field[e] : 1.0, TnI, accurate, R_e + (int64_t)m * e,
               K_e ? K_e + (int64_t)m * m * e : 0);
  }
}

/* 2-node traction lines in 2-D (neumann_weak + isoparametric_surface_element_galerkin,
   models.py:744-780, :1723-1851): R_ai = -sum_q N_a t_i w_q |dX/dxi| with 2 Gauss points,
   i.e. -t_i |x_1 - x_0| / 2 per node; R_e (n_l x 4) */
void orc_neumann_lines(int64_t n_l, const int64_t* lines, const double* coords, double tx, double ty, double* R_e) {
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < n_l; ++e) {
    const double* x0 = coords + 2 * lines[2 * e];
    const double* x1 = coords + 2 * lines[2 * e + 1];
    const double L = sqrt((x1[0] - x0[0]) * (x1[0] - x0[0]) + (x1[1] - x0[1]) * (x1[1] - x0[1]));
    R_e[4 * e + 0] = -0.5 * L * tx;
    R_e[4 * e + 1] = -0.5 * L * ty;
    R_e[4 * e + 2] = -0.5 * L * tx;
    R_e[4 * e + 3] = -0.5 * L * ty;
  }
}

/* R[conn[e,a] ndof + c] += R_e[e, a ndof + c] (serial: the element order of the reference's
   scatter-add, assembler.py:331-436) */
void orc_scatter(int64_t n_e, int nen, int ndof, const int64_t* conn, const double* R_e, double* R) {
  for (int64_t e = 0; e < n_e; ++e)
    for (int a = 0; a < nen; ++a)
      for (int c = 0; c < ndof; ++c) R[conn[nen * e + a] * ndof + c] += R_e[(int64_t)nen * ndof * e + ndof * a + c];
}
