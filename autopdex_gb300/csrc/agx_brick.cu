// Uniform structured brick grids: the backward-Euler heat model (models.py:1272-1357 with the
// integrand of examples/heat_conduction/maze_backward_euler.py, k = k0 + k2 T^2) assembled
// without the generic element kernel's per-point geometry and slot scatter.
//
// A HEX8 set that is the mesher's nx x ny x nz brick grid (node (i, j, k) at
// (i (ny + 1) + j)(nz + 1) + k, element (i ny + j) nz + k, local nodes in the mesher's order)
// whose nodes all lie on one lattice x0 + i e1 + j e2 + k e3 has one constant Jacobian
// J = [e1 | e2 | e3] / 2.  With the 2 x 2 x 2 Gauss rule (weights 1) every integral then
// needs only M = (J^T J)^-1 and det J, and the trilinear shape functions factor into 1-D
// ones: at Gauss coordinate p (xi = (2p - 1) / sqrt 3) node coordinate i has value
// B(p, i) = (1 + (2i - 1) xi) / 2 (alpha when i == p, beta otherwise) and derivative
// D(i) = (2i - 1) / 2.
//
// brick_heat_be_residual (float64): one thread per element.  Values and reference gradients
// at the 8 Gauss points by sum factorisation (one 1-D contraction per direction), the flux
// det k(T) M grad_xi T and its transposed contractions back to the 8 nodes; the mass term
// det rho_c / dt (T - T_n), linear, as the 1-D Gauss mass matrix applied per direction; added
// to R with reductions.  About a quarter of the float64 operations of the per-point
// evaluation, which is what bounds this pass on a GPU whose float64 rate is a fraction of its
// float32 rate.
//
// brick_heat_be_tangent (float32): one thread per node row, atomic-free, on a float32 copy of
// the DOFs.  The row of node
// (I, J, K) gathers the matrices of its up to 8 elements (each recomputed from the element's
// nodal values) into the 27-entry stencil, deletes prescribed columns (identity row at a
// prescribed node), writes 1 / diagonal, and the 128 rows of a block leave through shared
// memory as one contiguous, coalesced range of the values array (the rows of consecutive
// nodes are consecutive; an in-range stencil in (di, dj, dk) order is the row's sorted
// column order).
#include "agx_common.cuh"

namespace {

constexpr double kGa = 0.78867513459481288225;  // (1 + 1/sqrt(3)) / 2
constexpr double kGb = 0.21132486540518711775;  // (1 - 1/sqrt(3)) / 2

template <typename T>
__device__ __forceinline__ constexpr T bv(int p, int i) {
  return p == i ? (T)kGa : (T)kGb;
}
template <typename T>
__device__ __forceinline__ constexpr T dv(int i) {
  return i ? T(0.5) : T(-0.5);
}

struct BrickParams {
  double M[6];  // M00 M01 M02 M11 M12 M22 of (J^T J)^-1
  double det;   // det J (the Gauss weights are 1)
  double k0, k2, mass;  // k = k0 + k2 T^2; mass = rho_c / dt
};

// values F[p][q][r] at the Gauss points of a nodal field f[i][j][k]
template <typename T>
__device__ __forceinline__ void interp(const T (&f)[2][2][2], T (&F)[2][2][2]) {
  T a[2][2][2], b[2][2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int r = 0; r < 2; ++r) a[i][j][r] = bv<T>(r, 0) * f[i][j][0] + bv<T>(r, 1) * f[i][j][1];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int r = 0; r < 2; ++r) b[i][q][r] = bv<T>(q, 0) * a[i][0][r] + bv<T>(q, 1) * a[i][1][r];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int r = 0; r < 2; ++r) F[p][q][r] = bv<T>(p, 0) * b[0][q][r] + bv<T>(p, 1) * b[1][q][r];
}

// reference gradient at the Gauss points: d/dxi at (p, q, r) depends on (q, r) only, etc.
//   gx[q][r] = sum_jk B(q,j) B(r,k) (f[1][j][k] - f[0][j][k]) / 2, gy[p][r], gz[p][q] alike
template <typename T>
__device__ __forceinline__ void rgrad(const T (&f)[2][2][2], T (&gx)[2][2], T (&gy)[2][2], T (&gz)[2][2]) {
  T dx[2][2], dy[2][2], dz[2][2];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      dx[u][v] = T(0.5) * (f[1][u][v] - f[0][u][v]);  // (j, k)
      dy[u][v] = T(0.5) * (f[u][1][v] - f[u][0][v]);  // (i, k)
      dz[u][v] = T(0.5) * (f[u][v][1] - f[u][v][0]);  // (i, j)
    }
  auto two = [](const T (&d)[2][2], T (&g)[2][2]) {
    T a[2][2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int s = 0; s < 2; ++s) a[u][s] = bv<T>(s, 0) * d[u][0] + bv<T>(s, 1) * d[u][1];
#pragma unroll
    for (int t = 0; t < 2; ++t)
#pragma unroll
      for (int s = 0; s < 2; ++s) g[t][s] = bv<T>(t, 0) * a[0][s] + bv<T>(t, 1) * a[1][s];
  };
  two(dx, gx);
  two(dy, gy);
  two(dz, gz);
}

// transposed contractions: out[a][b][c] = sum_pqr B(p,a) B(q,b) B(r,c) F[p][q][r], and
// S[u][v] = sum_st B(s,u) B(t,v) H[s][t]
template <typename T>
__device__ __forceinline__ void tinterp(const T (&F)[2][2][2], T (&out)[2][2][2]) {
  T c1[2][2][2], c2[2][2][2];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int r = 0; r < 2; ++r) c1[a][q][r] = bv<T>(0, a) * F[0][q][r] + bv<T>(1, a) * F[1][q][r];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int r = 0; r < 2; ++r) c2[a][b][r] = bv<T>(0, b) * c1[a][0][r] + bv<T>(1, b) * c1[a][1][r];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 2; ++c) out[a][b][c] = bv<T>(0, c) * c2[a][b][0] + bv<T>(1, c) * c2[a][b][1];
}

template <typename T>
__device__ __forceinline__ void back2(const T (&H)[2][2], T (&S)[2][2]) {
  T a[2][2];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int t = 0; t < 2; ++t) a[u][t] = bv<T>(0, u) * H[0][t] + bv<T>(1, u) * H[1][t];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) S[u][v] = bv<T>(0, v) * a[u][0] + bv<T>(1, v) * a[u][1];
}

// the 1-D Gauss mass matrix B^T B = [[2, 1], [1, 2]] / 3
__device__ __forceinline__ constexpr float m1(int i, int j) { return i == j ? 2.0f / 3.0f : 1.0f / 3.0f; }

// DIAG: J^T J diagonal (an axis-aligned lattice), so M grad_xi T needs 3 products, not 9
template <bool DIAG>
__global__ void __launch_bounds__(256)
brick_heat_be_residual(int nx, int ny, int nz, const double* __restrict__ u, const double* __restrict__ un,
                       BrickParams bp, double* __restrict__ R) {
  const int64_t n_e = (int64_t)nx * ny * nz;
  const int64_t sa = (int64_t)(ny + 1) * (nz + 1), sb = nz + 1;
  const double M00 = bp.M[0], M01 = bp.M[1], M02 = bp.M[2], M11 = bp.M[3], M12 = bp.M[4], M22 = bp.M[5];
  const double k0d = bp.det * bp.k0, k2d = bp.det * bp.k2;
  // the mass term is linear: det mass (M1 x M1 x M1) (T - T_n) with the 1-D Gauss mass matrix
  // M1 = B^T B = [[2, 1], [1, 2]] / 3, applied as (x_c + x_0 + x_1) per direction and 1/27 at the end
  const double mdet = bp.det * bp.mass / 27.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_e; e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % nz);
    const int64_t ij = e / nz;
    const int j = (int)(ij % ny), i = (int)(ij / ny);
    const int64_t n0 = i * sa + j * sb + k;
    double t[2][2][2], d[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int64_t idx = n0 + a * sa + b * sb + c;
          t[a][b][c] = u[idx];
          d[a][b][c] = t[a][b][c] - un[idx];
        }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const double s2 = d[a][b][0] + d[a][b][1];
        d[a][b][0] += s2;
        d[a][b][1] += s2;
      }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const double s2 = d[a][0][c] + d[a][1][c];
        d[a][0][c] += s2;
        d[a][1][c] += s2;
      }
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const double s2 = d[0][b][c] + d[1][b][c];
        d[0][b][c] += s2;
        d[1][b][c] += s2;
      }
    double Tq[2][2][2], gx[2][2], gy[2][2], gz[2][2];
    interp(t, Tq);
    rgrad(t, gx, gy, gz);
    // per Gauss point the flux h = det k M grad_xi T, summed over the point coordinate that its
    // test-function contraction does not need
    double Hx[2][2], Hy[2][2], Hz[2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) Hx[a][b] = Hy[a][b] = Hz[a][b] = 0.0;
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const double T0 = Tq[p][q][r];
          const double kd = k0d + k2d * T0 * T0;
          const double g0 = gx[q][r], g1 = gy[p][r], g2 = gz[p][q];
          if constexpr (DIAG) {
            Hx[q][r] += kd * (M00 * g0);
            Hy[p][r] += kd * (M11 * g1);
            Hz[p][q] += kd * (M22 * g2);
          } else {
            Hx[q][r] += kd * (M00 * g0 + M01 * g1 + M02 * g2);
            Hy[p][r] += kd * (M01 * g0 + M11 * g1 + M12 * g2);
            Hz[p][q] += kd * (M02 * g0 + M12 * g1 + M22 * g2);
          }
        }
    // R[a][b][c] = mass part + D(a) Sx[b][c] + D(b) Sy[a][c] + D(c) Sz[a][b]
    double Sx[2][2], Sy[2][2], Sz[2][2];
    back2(Hx, Sx);  // [b][c]
    back2(Hy, Sy);  // [a][c]
    back2(Hz, Sz);  // [a][b]
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
          const double v = mdet * d[a][b][cc] + dv<double>(a) * Sx[b][cc] + dv<double>(b) * Sy[a][cc] +
                           dv<double>(cc) * Sz[a][b];
          atomicAdd(R + n0 + a * sa + b * sb + cc, v);
        }
  }
}

constexpr int kRowBlock = 128;  // node rows per block of the tangent kernel

__global__ void __launch_bounds__(256) dofs_to_float(int64_t n, const double* __restrict__ u, float* __restrict__ f) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    f[i] = (float)u[i];
}

// u: the DOFs rounded to float32 once (a float64 load and conversion per use would run on the
// float64 pipe: 64 per row)
template <bool DIAG>
__global__ void __launch_bounds__(kRowBlock)
brick_heat_be_tangent(int nx, int ny, int nz, const float* __restrict__ u, BrickParams bp,
                      const uint8_t* __restrict__ dmask, const int32_t* __restrict__ rowptr, float* __restrict__ vals,
                      float* __restrict__ dinv) {
  __shared__ float stage[kRowBlock * 27];
  const int64_t NY = ny + 1, NZ = nz + 1;
  const int64_t sa = NY * NZ, sb = NZ;
  const int64_t n_nodes = (int64_t)(nx + 1) * sa;
  const int64_t p0 = (int64_t)blockIdx.x * kRowBlock;
  const int64_t p = p0 + threadIdx.x;
  const float M00 = (float)bp.M[0], M01 = (float)bp.M[1], M02 = (float)bp.M[2], M11 = (float)bp.M[3],
              M12 = (float)bp.M[4], M22 = (float)bp.M[5];
  const float det = (float)bp.det, k0 = (float)bp.k0, k2 = (float)bp.k2, mass = (float)bp.mass;
  const int32_t rp0 = rowptr[p0];
  if (p < n_nodes) {
    const int K = (int)(p % NZ);
    const int64_t ij = p / NZ;
    const int J = (int)(ij % NY), I = (int)(ij / NY);
    float v[27];
#pragma unroll
    for (int s = 0; s < 27; ++s) v[s] = 0.0f;
    // the elements with this node as local node (di, dj, dk): origin (I - di, J - dj, K - dk)
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
      for (int dj = 0; dj < 2; ++dj)
#pragma unroll
        for (int dk = 0; dk < 2; ++dk) {
          const int ei = I - di, ej = J - dj, ek = K - dk;
          if (ei < 0 || ei >= nx || ej < 0 || ej >= ny || ek < 0 || ek >= nz) continue;
          const int64_t n0 = ei * sa + ej * sb + ek;
          float t[2][2][2];
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
              for (int c = 0; c < 2; ++c) t[a][b][c] = __ldg(u + n0 + a * sa + b * sb + c);
          float Tq[2][2][2], gx[2][2], gy[2][2], gz[2][2];
          interp(t, Tq);
          rgrad(t, gx, gy, gz);
          // row a = (di, dj, dk) of the element matrix, column b = (mi, mj, mk):
          //   sum_q [k_q (M grad_xi N_a).grad_xi N_b + det dk_q (M grad_xi N_a).grad_xi T N_b]
          //   + det mass (M1 x M1 x M1)_ab,
          // the Gauss sums as the test-function contractions of the residual: W collects
          // k_q M grad_xi N_a per point coordinate pair, c the N_b coefficients
          float Wx[2][2], Wy[2][2], Wz[2][2], c[2][2][2];
#pragma unroll
          for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int w2 = 0; w2 < 2; ++w2) Wx[u][w2] = Wy[u][w2] = Wz[u][w2] = 0.0f;
#pragma unroll
          for (int pp = 0; pp < 2; ++pp)
#pragma unroll
            for (int q = 0; q < 2; ++q)
#pragma unroll
              for (int r = 0; r < 2; ++r) {
                const float ga0 = dv<float>(di) * bv<float>(q, dj) * bv<float>(r, dk);
                const float ga1 = bv<float>(pp, di) * dv<float>(dj) * bv<float>(r, dk);
                const float ga2 = bv<float>(pp, di) * bv<float>(q, dj) * dv<float>(dk);
                float m0, m1_, m2;  // M grad_xi N_a
                if constexpr (DIAG) {
                  m0 = M00 * ga0, m1_ = M11 * ga1, m2 = M22 * ga2;
                } else {
                  m0 = M00 * ga0 + M01 * ga1 + M02 * ga2;
                  m1_ = M01 * ga0 + M11 * ga1 + M12 * ga2;
                  m2 = M02 * ga0 + M12 * ga1 + M22 * ga2;
                }
                const float T0 = Tq[pp][q][r];
                const float kq = det * (k0 + k2 * T0 * T0);
                Wx[q][r] += kq * m0;
                Wy[pp][r] += kq * m1_;
                Wz[pp][q] += kq * m2;
                c[pp][q][r] = det * 2.0f * k2 * T0 * (m0 * gx[q][r] + m1_ * gy[pp][r] + m2 * gz[pp][q]);
              }
          float Kc[2][2][2], Sx[2][2], Sy[2][2], Sz[2][2];
          tinterp(c, Kc);
          back2(Wx, Sx);  // [mj][mk]
          back2(Wy, Sy);  // [mi][mk]
          back2(Wz, Sz);  // [mi][mj]
          const float md = det * mass;
          float row[8];
#pragma unroll
          for (int mi = 0; mi < 2; ++mi)
#pragma unroll
            for (int mj = 0; mj < 2; ++mj)
#pragma unroll
              for (int mk = 0; mk < 2; ++mk)
                row[4 * mi + 2 * mj + mk] = Kc[mi][mj][mk] + dv<float>(mi) * Sx[mj][mk] + dv<float>(mj) * Sy[mi][mk] +
                                            dv<float>(mk) * Sz[mi][mj] +
                                            md * (m1(di, mi) * m1(dj, mj) * m1(dk, mk));
#pragma unroll
          for (int mi = 0; mi < 2; ++mi)
#pragma unroll
            for (int mj = 0; mj < 2; ++mj)
#pragma unroll
              for (int mk = 0; mk < 2; ++mk)
                v[(mi - di + 1) * 9 + (mj - dj + 1) * 3 + (mk - dk + 1)] += row[4 * mi + 2 * mj + mk];
        }
    // prescribed nodes: identity row; prescribed columns deleted
    if (dmask[p] & 1u) {
#pragma unroll
      for (int s = 0; s < 27; ++s) v[s] = 0.0f;
      v[13] = 1.0f;
    } else {
#pragma unroll
      for (int oi = -1; oi <= 1; ++oi)
#pragma unroll
        for (int oj = -1; oj <= 1; ++oj)
#pragma unroll
          for (int ok = -1; ok <= 1; ++ok) {
            const int ii = I + oi, jj = J + oj, kk = K + ok;
            if (ii < 0 || ii > nx || jj < 0 || jj > ny || kk < 0 || kk > nz) continue;
            if (__ldg(dmask + ii * sa + jj * sb + kk) & 1u) v[(oi + 1) * 9 + (oj + 1) * 3 + ok + 1] = 0.0f;
          }
    }
    dinv[p] = v[13] != 0.0f ? __frcp_rn(v[13]) : 0.0f;
    // the in-range entries in (oi, oj, ok) order, staged at this row's offset in the block
    float* sr = stage + (rowptr[p] - rp0);
    int w = 0;
#pragma unroll
    for (int oi = -1; oi <= 1; ++oi)
#pragma unroll
      for (int oj = -1; oj <= 1; ++oj)
#pragma unroll
        for (int ok = -1; ok <= 1; ++ok) {
          const int ii = I + oi, jj = J + oj, kk = K + ok;
          if (ii < 0 || ii > nx || jj < 0 || jj > ny || kk < 0 || kk > nz) continue;
          sr[w++] = v[(oi + 1) * 9 + (oj + 1) * 3 + ok + 1];
        }
  }
  __syncthreads();
  const int64_t pend = p0 + kRowBlock < n_nodes ? p0 + kRowBlock : n_nodes;
  const int32_t total = rowptr[pend] - rp0;
  for (int s = threadIdx.x; s < total; s += kRowBlock) vals[(int64_t)rp0 + s] = stage[s];
}

BrickParams brick_params(const agx_element_set& s) {
  BrickParams bp;
  for (int i = 0; i < 6; ++i) bp.M[i] = s.brick_m[i];
  bp.det = s.brick_det;
  bp.k0 = s.params[0];
  bp.k2 = s.params[1];
  bp.mass = s.params[2] / s.params[3];
  return bp;
}

}  // namespace

bool agx_brick_heat_be(const agx_context* ctx, const agx_element_set& s) {
  return s.brick_n[0] > 0 && s.brick_uniform && s.model == AGX_MODEL_HEAT_BE && s.elem_type == AGX_HEX8 &&
         s.ngauss == 2 && ctx->ndof == 1 && s.d_node_field != nullptr && s.params[3] != 0.0;
}

void agx_launch_brick_residual(agx_context* ctx, const agx_element_set& s, const double* dofs, double* R) {
  const int64_t n_e = (int64_t)s.brick_n[0] * s.brick_n[1] * s.brick_n[2];
  const bool diag = s.brick_m[1] == 0.0 && s.brick_m[2] == 0.0 && s.brick_m[4] == 0.0;
  if (diag)
    brick_heat_be_residual<true><<<agx_grid(ctx, n_e), 256, 0, ctx->stream>>>(
        s.brick_n[0], s.brick_n[1], s.brick_n[2], dofs, s.d_node_field, brick_params(s), R);
  else
    brick_heat_be_residual<false><<<agx_grid(ctx, n_e), 256, 0, ctx->stream>>>(
        s.brick_n[0], s.brick_n[1], s.brick_n[2], dofs, s.d_node_field, brick_params(s), R);
  ctx->n_launches += 1;
}

void agx_launch_brick_tangent(agx_context* ctx, const agx_element_set& s, const double* dofs, float* vals,
                              float* dinv) {
  const int64_t n = ctx->n_nodes;
  dofs_to_float<<<agx_grid(ctx, n), 256, 0, ctx->stream>>>(n, dofs, ctx->f_dofs32);
  const unsigned grid = (unsigned)((n + kRowBlock - 1) / kRowBlock);
  if (s.brick_m[1] == 0.0 && s.brick_m[2] == 0.0 && s.brick_m[4] == 0.0)
    brick_heat_be_tangent<true><<<grid, kRowBlock, 0, ctx->stream>>>(s.brick_n[0], s.brick_n[1], s.brick_n[2],
                                                                     ctx->f_dofs32, brick_params(s), ctx->d_dmask_node,
                                                                     ctx->d_rowptr, vals, dinv);
  else
    brick_heat_be_tangent<false><<<grid, kRowBlock, 0, ctx->stream>>>(s.brick_n[0], s.brick_n[1], s.brick_n[2],
                                                                      ctx->f_dofs32, brick_params(s), ctx->d_dmask_node,
                                                                      ctx->d_rowptr, vals, dinv);
  ctx->n_launches += 2;
}
