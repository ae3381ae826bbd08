// Element residual / tangent assembly for the built-in Q1 models.
//
// Replaces the per-element AD of AutoPDEx (jacrev / jacfwd(jacrev) under vmap / lax.map,
// assembler.py:1064-1149, :1216-1306, :1310-1389) and the scatter-adds of _get_residual
// (assembler.py:331-436) and of the BCOO tangent (assembler.py:1142-1148, summed later by
// scipy_assembling, solver.py:1180-1222).
//
// Mapping to the GPU: a group of NEN consecutive lanes handles one element, lane a owning
// element node a.  Per Gauss point each lane evaluates its own shape function N_a and
// physical gradient g_a = dN_a/dxi J^-1 (the rule of fem_iso_line_quad_brick with
// overwrite_diff=True, spaces.py:12162-12190); element sums (Jacobian, field values and
// gradients at the point) are butterfly reductions inside the group, and the values of
// the other nodes needed for row a of the tangent are read from a per-warp shared-memory
// slab.  Lane a accumulates residual entries R_a and tangent row K_ab in registers and adds
// them into the residual vector and the node-block CSR values at positions precomputed by
// agx_build_pattern.  Entries of prescribed rows/columns are skipped (Dirichlet row and
// column deletion of scipy_assembling); prescribed diagonals are set to one beforehand.
//
// The element formulas are the closed forms of what the reference differentiates:
//   potential 1/2 k |grad u|^2 - s u        R_a = k grad u . g_a - s N_a,  K_ab = k g_a . g_b
//   neo-Hooke (Ciarlet, models.py:1122-1146), P = mu F + c F^-T, c = lam/2 (J^2-1) - mu
//     R_a,i = P_iJ g_a,J
//     K_ab,ik = mu (g_a.g_b) d_ik - c h_b,i h_a,k + lam J^2 h_a,i h_b,k,  h = F^-T g
//   backward-Euler heat rho_c (T-T_n)/dt v + k(T) grad T . grad v, k = k0 + k2 T^2
//     K_ab = rho_c/dt N_a N_b + k g_a.g_b + k'(T) N_b grad T . g_a   (non-symmetric)
//   Neumann traction (models.py:744-780, :1818-1827)  R_a,i = -N_a t_i |dX/dxi|
// all times the Gauss weight and det J; the oracle derives the same quantities by AD.
#include <type_traits>

#include "agx_common.cuh"

namespace {

template <int ET>
struct ElemTraits;
// GROUP: lanes per element (a power of two >= NEN; lanes a >= NEN carry zero shape functions)
template <>
struct ElemTraits<AGX_QUAD4> {
  static constexpr int RDIM = 2, NEN = 4, GROUP = 4;
};
template <>
struct ElemTraits<AGX_HEX8> {
  static constexpr int RDIM = 3, NEN = 8, GROUP = 8;
};
template <>
struct ElemTraits<AGX_LINE2> {
  static constexpr int RDIM = 1, NEN = 2, GROUP = 2;
};
template <>
struct ElemTraits<AGX_QUAD9> {
  static constexpr int RDIM = 2, NEN = 9, GROUP = 16;
};
template <>
struct ElemTraits<AGX_LINE3> {
  static constexpr int RDIM = 1, NEN = 3, GROUP = 4;
};
template <>
struct ElemTraits<AGX_TRI3> {
  static constexpr int RDIM = 2, NEN = 3, GROUP = 4;
};
template <>
struct ElemTraits<AGX_TRI6> {
  static constexpr int RDIM = 2, NEN = 6, GROUP = 8;
};
template <>
struct ElemTraits<AGX_TET4> {
  static constexpr int RDIM = 3, NEN = 4, GROUP = 4;
};
template <>
struct ElemTraits<AGX_HEX27> {
  static constexpr int RDIM = 3, NEN = 27, GROUP = 32;
};
template <>
struct ElemTraits<AGX_TET10> {
  static constexpr int RDIM = 3, NEN = 10, GROUP = 16;
};
template <int ET>
__host__ __device__ constexpr bool is_simplex() {
  return ET == AGX_TRI3 || ET == AGX_TRI6 || ET == AGX_TET4 || ET == AGX_TET10;
}
template <int ET>
__host__ __device__ constexpr int space_dim() {
  return (ET == AGX_HEX8 || ET == AGX_HEX27 || ET == AGX_TET4 || ET == AGX_TET10) ? 3 : 2;
}

// integration points of a simplex set (reference coordinates and weights), passed by value
struct QuadTable {
  int n;
  double x[AGX_MAX_QPOINTS][3];
  double w[AGX_MAX_QPOINTS];
};

// 2-point Gauss-Legendre on [-1, 1] from the [0, 1] rule of seeder.py:382-386 mapped as
// seeder.py:1053-1058; weights 2 * 0.5 = 1.
__device__ __forceinline__ double gauss_point(int i) {
  return i ? (2.0 * 0.7886751345948129 - 1.0) : (2.0 * 0.21132486540518713 - 1.0);
}

// n-point rule (n = 2 or 3) on [-1, 1]: the [0, 1] points and weights of seeder.py:324-386
// mapped as seeder.py:1053-1058 (x -> 2 x - 1, w -> 2 w), formed in float64 at compile time
// and rounded to T once, so that a float32 pass selects constants instead of converting
template <typename T>
__device__ __forceinline__ void gauss_rule(int n, int i, T& x, T& w) {
  if (n == 3) {
    x = i == 0 ? T(2.0 * 0.1127016653792583 - 1.0) : (i == 1 ? T(2.0 * 0.5 - 1.0) : T(2.0 * 0.8872983346207417 - 1.0));
    w = i == 1 ? T(2.0 * 0.44444444444444453) : T(2.0 * 0.2777777777777777);
  } else {
    x = i ? T(2.0 * 0.7886751345948129 - 1.0) : T(2.0 * 0.21132486540518713 - 1.0);
    w = T(1);
  }
}

// 1-D quadratic Lagrange basis on nodes -1, 0, +1 (index 0, 1, 2) and its derivative
template <typename T>
__device__ __forceinline__ void lagrange2(int k, T x, T& l, T& dl) {
  if (k == 0) {
    l = T(0.5) * x * (x - T(1));
    dl = x - T(0.5);
  } else if (k == 1) {
    l = T(1) - x * x;
    dl = T(-2) * x;
  } else {
    l = T(0.5) * x * (x + T(1));
    dl = x + T(0.5);
  }
}

// reference-node sign of node a in direction d (node orders of spaces.py:1913-1922,
// :12057-12081, :356-358)
template <int ET>
__device__ __forceinline__ int node_sign(int a, int d) {
  if (ET == AGX_LINE2 || ET == AGX_LINE3) return a ? 1 : -1;
  if (d == 0) return (a & 3) == 1 || (a & 3) == 2 ? 1 : -1;
  if (d == 1) return (a & 3) >= 2 ? 1 : -1;
  return a >= 4 ? 1 : -1;
}

// N_a(xi) and dN_a/dxi of the element's node a (node orders of spaces.py:1913-1922,
// :12057-12081, :356-358 and the quadratic orders of fem_iso_line_quad_brick)
template <int ET, typename T>
__device__ __forceinline__ void shape(int a, const T* xi, T& Na, T* dN) {
  if constexpr (ET == AGX_QUAD9) {
    // corners (-1,-1) (1,-1) (1,1) (-1,1), mid-sides (0,-1) (1,0) (0,1) (-1,0), centre:
    // x indices 0 2 2 0 1 2 1 0 1 and y indices 0 0 2 2 0 1 2 1 1, two bits per node
    constexpr unsigned IX = 0u | 2u << 2 | 2u << 4 | 0u << 6 | 1u << 8 | 2u << 10 | 1u << 12 | 0u << 14 | 1u << 16;
    constexpr unsigned IY = 0u | 0u << 2 | 2u << 4 | 2u << 6 | 0u << 8 | 1u << 10 | 2u << 12 | 1u << 14 | 1u << 16;
    T lx, dlx, ly, dly;
    lagrange2<T>((int)((IX >> (2 * a)) & 3u), xi[0], lx, dlx);
    lagrange2<T>((int)((IY >> (2 * a)) & 3u), xi[1], ly, dly);
    Na = lx * ly;
    dN[0] = dlx * ly;
    dN[1] = lx * dly;
  } else if constexpr (ET == AGX_TRI3) {
    // N = 1 - xi - eta, xi, eta (the 3-node case of fem_iso_line_tri_tet, n_dim 2)
    Na = a == 0 ? T(1) - xi[0] - xi[1] : (a == 1 ? xi[0] : xi[1]);
    dN[0] = a == 0 ? T(-1) : (a == 1 ? T(1) : T(0));
    dN[1] = a == 0 ? T(-1) : (a == 2 ? T(1) : T(0));
  } else if constexpr (ET == AGX_TET4) {
    // N = 1 - xi - eta - zeta, xi, eta, zeta (the 4-node case, n_dim 3)
    Na = a == 0 ? T(1) - xi[0] - xi[1] - xi[2] : (a == 1 ? xi[0] : (a == 2 ? xi[1] : xi[2]));
#pragma unroll
    for (int d = 0; d < 3; ++d) dN[d] = a == 0 ? T(-1) : (a == d + 1 ? T(1) : T(0));
  } else if constexpr (ET == AGX_HEX27) {
    // tensor products of the 1-D quadratic basis (index 0: -1, 1: 0, 2: +1); two bits per
    // node and direction in the node order of the 27-node case
    constexpr unsigned long long IX = 0x15582819192828ull, IY = 0x1585a06464a0a0ull, IZ = 0x185555aa00aa00ull;
    T lx, dlx, ly, dly, lz, dlz;
    lagrange2<T>((int)((IX >> (2 * a)) & 3ull), xi[0], lx, dlx);
    lagrange2<T>((int)((IY >> (2 * a)) & 3ull), xi[1], ly, dly);
    lagrange2<T>((int)((IZ >> (2 * a)) & 3ull), xi[2], lz, dlz);
    Na = lx * ly * lz;
    dN[0] = dlx * ly * lz;
    dN[1] = lx * dly * lz;
    dN[2] = lx * ly * dlz;
  } else if constexpr (ET == AGX_TET10) {
    // the 10-node case in barycentric form, L0 = 1 - xi - eta - zeta, L1..3 = xi, eta, zeta:
    // corners L_k (2 L_k - 1), edges 4 L_i L_j for (i, j) = (0,1) (1,2) (0,2) (0,3) (1,3) (2,3)
    auto L = [&](int k) { return k == 0 ? T(1) - xi[0] - xi[1] - xi[2] : (k == 1 ? xi[0] : (k == 2 ? xi[1] : xi[2])); };
    auto dL = [](int k, int d) { return k == 0 ? T(-1) : (k == d + 1 ? T(1) : T(0)); };  // dL_k / dxi_d
    if (a < 4) {
      const T l = L(a);
      Na = l * (T(2) * l - T(1));
#pragma unroll
      for (int d = 0; d < 3; ++d) dN[d] = (T(4) * l - T(1)) * dL(a, d);
    } else {
      constexpr unsigned EI = 0u | 1u << 4 | 0u << 8 | 0u << 12 | 1u << 16 | 2u << 20;
      constexpr unsigned EJ = 1u | 2u << 4 | 2u << 8 | 3u << 12 | 3u << 16 | 3u << 20;
      const int i = (int)((EI >> (4 * (a - 4))) & 15u), j = (int)((EJ >> (4 * (a - 4))) & 15u);
      const T li = L(i), lj = L(j);
      Na = T(4) * li * lj;
#pragma unroll
      for (int d = 0; d < 3; ++d) dN[d] = T(4) * (li * dL(j, d) + lj * dL(i, d));
    }
  } else if constexpr (ET == AGX_TRI6) {
    // the 6-node case, in barycentric form with L0 = 1 - xi - eta, L1 = xi, L2 = eta:
    // corners L_i (2 L_i - 1), mid-sides 4 L0 L1, 4 L1 L2, 4 L2 L0
    const T L0 = T(1) - xi[0] - xi[1], L1 = xi[0], L2 = xi[1];
    // dL/dxi = (-1, 1, 0), dL/deta = (-1, 0, 1)
    if (a == 0) {
      Na = L0 * (T(2) * L0 - T(1));
      dN[0] = dN[1] = -(T(4) * L0 - T(1));
    } else if (a == 1) {
      Na = L1 * (T(2) * L1 - T(1));
      dN[0] = T(4) * L1 - T(1);
      dN[1] = T(0);
    } else if (a == 2) {
      Na = L2 * (T(2) * L2 - T(1));
      dN[0] = T(0);
      dN[1] = T(4) * L2 - T(1);
    } else if (a == 3) {
      Na = T(4) * L0 * L1;
      dN[0] = T(4) * (L0 - L1);
      dN[1] = -T(4) * L1;
    } else if (a == 4) {
      Na = T(4) * L1 * L2;
      dN[0] = T(4) * L2;
      dN[1] = T(4) * L1;
    } else {
      Na = T(4) * L2 * L0;
      dN[0] = -T(4) * L2;
      dN[1] = T(4) * (L0 - L2);
    }
  } else if constexpr (ET == AGX_LINE3) {
    // end nodes -1, +1, then the middle node: indices 0 2 1
    T l, dl;
    lagrange2<T>(a == 0 ? 0 : (a == 1 ? 2 : 1), xi[0], l, dl);
    Na = l;
    dN[0] = dl;
  } else {
    constexpr int RD = ElemTraits<ET>::RDIM;
    T fac[RD];
#pragma unroll
    for (int d = 0; d < RD; ++d) fac[d] = (T(1) + T(node_sign<ET>(a, d)) * xi[d]) * T(0.5);
    Na = 1;
#pragma unroll
    for (int d = 0; d < RD; ++d) Na *= fac[d];
#pragma unroll
    for (int d = 0; d < RD; ++d) {
      T v = T(node_sign<ET>(a, d)) * T(0.5);
#pragma unroll
      for (int d2 = 0; d2 < RD; ++d2)
        if (d2 != d) v *= fac[d2];
      dN[d] = v;
    }
  }
}


template <int NEN, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = NEN / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T det2(const T (&m)[2][2]) { return m[0][0] * m[1][1] - m[0][1] * m[1][0]; }
template <typename T>
__device__ __forceinline__ T det3(const T (&m)[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
         m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}
// inverse by the adjugate (utility.py:706-770)
template <typename T, int D>
__device__ __forceinline__ T inverse(const T (&m)[D][D], T (&inv)[D][D]) {
  if constexpr (D == 2) {
    T d = det2(m), r = T(1) / d;
    inv[0][0] = m[1][1] * r; inv[0][1] = -m[0][1] * r;
    inv[1][0] = -m[1][0] * r; inv[1][1] = m[0][0] * r;
    return d;
  } else {
    T d = det3(m), r = T(1) / d;
    inv[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * r;
    inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * r;
    inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * r;
    inv[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * r;
    inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * r;
    inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * r;
    inv[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * r;
    inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * r;
    inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * r;
    return d;
  }
}

// Ciarlet neo-Hooke quantities (models.py:1122-1146) from the displacement gradient H = F - I,
// written without cancellation near F = I.  J - 1 = tr H + i2(H) + det H (i2 the sum of the
// principal 2 x 2 minors; plane strain: tr H + det H), and I - F^-T = (H^T + (i2 + det H) I -
// cof H) / J (plane strain: (H^T + det H I) / J), so that
//   P = mu (F - F^-T) + lam/2 (J^2 - 1) F^-T = mu (H + I - F^-T) + lam/2 (J-1)(J+1) F^-T.
// Forming J = det F and then J^2 - 1 loses |F| eps absolutely, which lam turns into a stress
// error of lam eps: with nu = 0.4999 (lam / mu = 5000) that rounding, not the solver, bounded the
// float64 Newton residual near 1e-6 of the load-step residual on Cook's membrane.  Returns J - 1
// and fills P, F^-1 (for the tangent) and J.
template <typename T, int D>
__device__ __forceinline__ T neo_hooke_stress(const T (&H)[D][D], T lam, T mu, T (&P)[D][D], T (&Fi)[D][D], T& Jdet) {
  T jm1, s;  // J - 1 and the scalar multiplying I in J (I - F^-T)
  T C[D][D];  // cofactor matrix of F (F^-T = C / J)
  if constexpr (D == 2) {
    const T dH = det2(H);
    jm1 = (H[0][0] + H[1][1]) + dH;
    s = dH;
    C[0][0] = T(1) + H[1][1]; C[0][1] = -H[1][0];
    C[1][0] = -H[0][1];       C[1][1] = T(1) + H[0][0];
  } else {
    const T i2 = (H[0][0] * H[1][1] - H[0][1] * H[1][0]) + (H[0][0] * H[2][2] - H[0][2] * H[2][0]) +
                 (H[1][1] * H[2][2] - H[1][2] * H[2][1]);
    const T dH = det3(H);
    jm1 = (H[0][0] + H[1][1] + H[2][2]) + (i2 + dH);
    s = i2 + dH;
    T F[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? T(1) : T(0));
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int i1 = (i + 1) % 3, i2_ = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        C[i][j] = F[i1][j1] * F[i2_][j2] - F[i1][j2] * F[i2_][j1];
      }
  }
  Jdet = T(1) + jm1;
  const T rJ = T(1) / Jdet;
  const T pl = lam * T(0.5) * jm1 * (T(2) + jm1);  // lam/2 (J^2 - 1)
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      Fi[j][i] = C[i][j] * rJ;  // F^-1 = C^T / J
      // cof H, the third term of J (I - F^-T) in 3-D: the cofactors of H
      T cofH = T(0);
      if constexpr (D == 3) {
        const int i1 = (i + 1) % 3, i2_ = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        cofH = H[i1][j1] * H[i2_][j2] - H[i1][j2] * H[i2_][j1];
      }
      const T m = (H[j][i] + (i == j ? s : T(0)) - cofH) * rJ;  // (I - F^-T)_ij
      P[i][j] = mu * (H[i][j] + m) + pl * C[i][j] * rJ;
    }
  return jm1;
}

struct ModelParams {
  double p[AGX_MAX_PARAMS];
};

template <int MODEL, int SDIM>
struct ModelTraits {
  static constexpr int NDOF = (MODEL == AGX_MODEL_NEO_HOOKE || MODEL == AGX_MODEL_NEUMANN) ? SDIM : 1;
  static constexpr bool HAS_K = MODEL != AGX_MODEL_NEUMANN;
  static constexpr int SLOTS = 1 + SDIM + (MODEL == AGX_MODEL_NEO_HOOKE ? SDIM : 0);  // N, g, h
};

// One kernel per (element type, model, arithmetic type, what to compute).  CB > 0: the
// tangent columns of nodes b0 .. b0 + CB - 1 only (a lane holds CB x NDOF x NDOF accumulators
// instead of NEN x NDOF x NDOF: the 27-node brick's neo-Hooke tangent row, 243 entries, is
// assembled in passes over column chunks, each recomputing the element's Gauss points).
template <int ET, int MODEL, typename T, bool DO_R, bool DO_K, int CB = 0>
__global__ void __launch_bounds__(AGX_BLOCK)
element_kernel(int64_t n_elem, const int32_t* __restrict__ conn, const int32_t* __restrict__ epos,
               const T* __restrict__ coords, const double* __restrict__ dofs,
               const T* __restrict__ elem_field, const double* __restrict__ node_field,
               const uint8_t* __restrict__ dmask_node, ModelParams mp, double* __restrict__ R,
               T* __restrict__ vals, int64_t nnzb, const double* __restrict__ geo, double* __restrict__ geo_out,
               int ng, const QuadTable qt, int b0 = 0) {
  using ET_ = ElemTraits<ET>;
  constexpr int RDIM = ET_::RDIM, NEN = ET_::NEN, GROUP = ET_::GROUP;
  constexpr int NCOL = (CB > 0 && CB < NEN) ? CB : NEN;  // tangent column nodes of this pass
  constexpr bool CHUNKED = NCOL < NEN;
  const int c0 = CHUNKED ? b0 : 0;
  // integration points per element: the simplex set's table, or the ng-point Gauss rule per direction
  const int NQ = is_simplex<ET>() ? qt.n : (RDIM == 1 ? ng : (RDIM == 2 ? ng * ng : ng * ng * ng));
  constexpr int SDIM = space_dim<ET>();
  using MT = ModelTraits<MODEL, SDIM>;
  constexpr int NDOF = MT::NDOF, SLOTS = MT::SLOTS;

  __shared__ T slab[AGX_BLOCK / 32][32][SLOTS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int a = lane % GROUP, gbase = lane - a;
  const bool act = a < NEN;   // lanes past the element's nodes carry zero shape functions
  const int ac = act ? a : 0;
  const int64_t total = ((n_elem * GROUP + 31) / 32) * 32;

  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total;
       L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e_raw = L / GROUP;
    const bool valid = e_raw < n_elem;
    const int64_t e = valid ? e_raw : (n_elem - 1);
    const int node = conn[e * NEN + ac];

    T xa[SDIM];
#pragma unroll
    for (int d = 0; d < SDIM; ++d) xa[d] = coords[(int64_t)node * SDIM + d];
    T ua[NDOF];
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
      ua[c] = (MODEL == AGX_MODEL_NEUMANN || dofs == nullptr) ? T(0) : (T)dofs[(int64_t)node * NDOF + c];
    T tna = 0;
    if constexpr (MODEL == AGX_MODEL_HEAT_BE) tna = (T)node_field[node];
    T ke = 1;
    if constexpr (MODEL == AGX_MODEL_HEAT_POTENTIAL) ke = elem_field ? elem_field[e] : T(1);
    // Lame parameters (models.py:955-956) formed in float64 and then rounded: in float32,
    // 1 - 2 nu loses four digits at nu = 0.4999
    T lam = 0, mu = 0;
    if constexpr (MODEL == AGX_MODEL_NEO_HOOKE) {
      const double E = mp.p[0], nu = mp.p[1];
      lam = (T)(E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
      mu = (T)(E / (2.0 * (1.0 + nu)));
    }

    double Ra[NDOF];
#pragma unroll
    for (int c = 0; c < NDOF; ++c) Ra[c] = 0.0;
    T K[DO_K ? NCOL : 1][DO_K ? NDOF : 1][DO_K ? NDOF : 1];
    if constexpr (DO_K) {
#pragma unroll
      for (int b = 0; b < NCOL; ++b)
#pragma unroll
        for (int i = 0; i < NDOF; ++i)
#pragma unroll
          for (int j = 0; j < NDOF; ++j) K[b][i][j] = 0;
    }

#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      // Gauss point q (first reference coordinate fastest, seeder.py:1046-1062), its weight,
      // and the shape function and reference derivatives of node a
      T xi[RDIM];
      T wq = 1;
      if constexpr (is_simplex<ET>()) {
#pragma unroll
        for (int d = 0; d < RDIM; ++d) xi[d] = (T)qt.x[q][d];
        wq = (T)qt.w[q];
      } else {
        int r = q;
#pragma unroll
        for (int d = 0; d < RDIM; ++d) {
          T x, w;
          gauss_rule(ng, r % ng, x, w);
          r /= ng;
          xi[d] = x;
          wq *= w;
        }
      }
      T Na, dN[RDIM];
      shape<ET, T>(ac, xi, Na, dN);
      if (!act) {
        Na = 0;
#pragma unroll
        for (int d = 0; d < RDIM; ++d) dN[d] = 0;
      }
      if constexpr (MODEL == AGX_MODEL_NEUMANN) {
        // line in 2-D: |G1 x E3| = |G1| (models.py:1818-1823)
        T G[SDIM];
#pragma unroll
        for (int i = 0; i < SDIM; ++i) G[i] = group_sum<GROUP>(xa[i] * dN[0]);
        T len = sqrt(G[0] * G[0] + G[1] * G[1]);
        if constexpr (DO_R) {
#pragma unroll
          for (int c = 0; c < NDOF; ++c) Ra[c] += -(double)(Na * (T)mp.p[c] * len) * wq;
        }
        continue;
      } else {
        // physical gradient g_a = dN_a/dxi J^-1 and w det J: from the float64 geometry cache
        // when one is given (uniform branch), else from the isoparametric Jacobian dX/dxi
        T ga[SDIM];
        T wdet;
        const int64_t grec = ((e * NQ + q) * NEN + ac) * (SDIM + 1);
        if (geo != nullptr) {
#pragma unroll
          for (int d = 0; d < SDIM; ++d) ga[d] = act ? (T)geo[grec + d] : T(0);
          wdet = (T)geo[grec + SDIM];
        } else {
          T Jm[SDIM][SDIM], Ji[SDIM][SDIM];
#pragma unroll
          for (int i = 0; i < SDIM; ++i)
#pragma unroll
            for (int j = 0; j < SDIM; ++j) Jm[i][j] = group_sum<GROUP>(xa[i] * dN[j]);
          wdet = inverse<T, SDIM>(Jm, Ji) * wq;
#pragma unroll
          for (int d = 0; d < SDIM; ++d) {
            T v = 0;
#pragma unroll
            for (int k = 0; k < SDIM; ++k) v += dN[k] * Ji[k][d];
            ga[d] = v;
          }
          if (geo_out != nullptr && valid && act) {
#pragma unroll
            for (int d = 0; d < SDIM; ++d) geo_out[grec + d] = (double)ga[d];
            geo_out[grec + SDIM] = (double)wdet;
          }
        }

        if constexpr (MODEL == AGX_MODEL_POISSON_SINCOS || MODEL == AGX_MODEL_HEAT_POTENTIAL ||
                      MODEL == AGX_MODEL_HEAT_BE) {
          T gu[SDIM];
#pragma unroll
          for (int d = 0; d < SDIM; ++d) gu[d] = group_sum<GROUP>(ua[0] * ga[d]);
          T gug = 0;
#pragma unroll
          for (int d = 0; d < SDIM; ++d) gug += gu[d] * ga[d];
          T kq = ke, dkq = 0, mass = 0, src = 0;
          if constexpr (MODEL == AGX_MODEL_POISSON_SINCOS) {
            if constexpr (DO_R) {
              T xq[SDIM];
#pragma unroll
              for (int d = 0; d < SDIM; ++d) xq[d] = group_sum<GROUP>(Na * xa[d]);
              T r1 = 0, r2 = 0;
#pragma unroll
              for (int d = 0; d < SDIM; ++d) {
                r1 += xq[d] * xq[d];
                T y = xq[d] - (T)mp.p[2 + d];
                r2 += y * y;
              }
              const T w = (T)mp.p[1];
              src = (T)mp.p[0] * (sin(w * r1) - cos(w * r2));
            }
          } else if constexpr (MODEL == AGX_MODEL_HEAT_POTENTIAL) {
            src = (T)mp.p[0];
          } else {  // HEAT_BE: params k0, k2, rho_c, dt
            const T Tq = group_sum<GROUP>(Na * ua[0]);
            const T Tn = group_sum<GROUP>(Na * tna);
            kq = (T)mp.p[0] + (T)mp.p[1] * Tq * Tq;
            dkq = T(2) * (T)mp.p[1] * Tq;
            mass = (T)mp.p[2] / (T)mp.p[3];
            src = -mass * (Tq - Tn);  // enters as -src * N_a
          }
          if constexpr (DO_R) Ra[0] += (double)(wdet * (kq * gug - src * Na));
          if constexpr (DO_K) {
            __syncwarp();
            slab[warp][lane][0] = Na;
#pragma unroll
            for (int d = 0; d < SDIM; ++d) slab[warp][lane][1 + d] = ga[d];
            __syncwarp();
#pragma unroll
            for (int bb = 0; bb < NCOL; ++bb) {
              const int b = c0 + bb;
              if (CHUNKED && b >= NEN) break;
              const T Nb = slab[warp][gbase + b][0];
              T gg = 0;
#pragma unroll
              for (int d = 0; d < SDIM; ++d) gg += ga[d] * slab[warp][gbase + b][1 + d];
              T kab = kq * gg;
              if constexpr (MODEL == AGX_MODEL_HEAT_BE) kab += mass * Na * Nb + dkq * Nb * gug;
              K[bb][0][0] += wdet * kab;
            }
          }
        } else if constexpr (MODEL == AGX_MODEL_NEO_HOOKE) {
          // displacement gradient and deformation gradient (plane strain: F33 = 1)
          T Hg[SDIM][SDIM];
#pragma unroll
          for (int i = 0; i < SDIM; ++i)
#pragma unroll
            for (int j = 0; j < SDIM; ++j) Hg[i][j] = group_sum<GROUP>(ua[i] * ga[j]);
          T Fi[SDIM][SDIM], P[SDIM][SDIM], Jdet;
          const T jm1 = neo_hooke_stress<T, SDIM>(Hg, lam, mu, P, Fi, Jdet);
          const T c = lam * T(0.5) * jm1 * (T(2) + jm1) - mu;
          T ha[SDIM];
#pragma unroll
          for (int i = 0; i < SDIM; ++i) {
            T v = 0;
#pragma unroll
            for (int j = 0; j < SDIM; ++j) v += Fi[j][i] * ga[j];  // (F^-T g)_i
            ha[i] = v;
          }
          if constexpr (DO_R) {
#pragma unroll
            for (int i = 0; i < SDIM; ++i) {
              T pg = 0;
#pragma unroll
              for (int j = 0; j < SDIM; ++j) pg += P[i][j] * ga[j];
              Ra[i] += (double)(wdet * pg);
            }
          }
          if constexpr (DO_K) {
            __syncwarp();
#pragma unroll
            for (int d = 0; d < SDIM; ++d) {
              slab[warp][lane][1 + d] = ga[d];
              slab[warp][lane][1 + SDIM + d] = ha[d];
            }
            __syncwarp();
            const T lj2 = lam * Jdet * Jdet;
#pragma unroll
            for (int bb = 0; bb < NCOL; ++bb) {
              const int b = c0 + bb;
              if (CHUNKED && b >= NEN) break;
              T gb[SDIM], hb[SDIM];
#pragma unroll
              for (int d = 0; d < SDIM; ++d) {
                gb[d] = slab[warp][gbase + b][1 + d];
                hb[d] = slab[warp][gbase + b][1 + SDIM + d];
              }
              T gg = 0;
#pragma unroll
              for (int d = 0; d < SDIM; ++d) gg += ga[d] * gb[d];
#pragma unroll
              for (int i = 0; i < SDIM; ++i)
#pragma unroll
                for (int k = 0; k < SDIM; ++k)
                  K[bb][i][k] += wdet * ((i == k ? mu * gg : T(0)) - c * hb[i] * ha[k] + lj2 * ha[i] * hb[k]);
            }
          }
        }
      }
    }

    // scatter into the residual and the pattern
    const unsigned dma = dmask_node[node];
    if constexpr (DO_R) {
      if (valid && act) {
#pragma unroll
        for (int c = 0; c < NDOF; ++c) atomicAdd(R + (int64_t)node * NDOF + c, Ra[c]);
      }
    }
    if constexpr (DO_K && MT::HAS_K) {
#pragma unroll
      for (int bb = 0; bb < NCOL; ++bb) {
        const int b = c0 + bb;
        if (CHUNKED && b >= NEN) break;
        const unsigned dmb = __shfl_sync(0xffffffffu, dma, gbase + b);
        if (valid && act) {
          // entry-major value planes: entry (i, j) of block pos at vals[(i ndof + j) nnzb + pos]
          T* blk = vals + epos[(e * NEN + a) * NEN + b];
#pragma unroll
          for (int i = 0; i < NDOF; ++i)
#pragma unroll
            for (int j = 0; j < NDOF; ++j)
              if (!((dma >> i) & 1u) && !((dmb >> j) & 1u))
                atomicAdd(blk + (int64_t)(i * NDOF + j) * nnzb, K[bb][i][j]);
        }
      }
    }
  }
}

// ---- atomic-free tangent of a structured quad grid (column sweep) -------------------------
// For a set that detect_structured_grid recognised and a scalar potential model (K_ab =
// k int g_a . g_b, symmetric), the tangent is written row by row and without atomics.  A warp
// owns a strip of GS_NODES = 31 node columns and a segment of node rows and walks down it:
// lane l computes the element to the right of node column c0 + l - 1 (lane 0 the element left
// of the strip), keeps the previous element row in registers, receives the left element's
// share of its node's row by one shuffle per entry, and writes the node's nine entries and
// its inverse diagonal once.  Coordinates, coefficients, Dirichlet flags and row pointers of
// the next row are requested before the current row is computed.  DRAM traffic is each of
// those once (plus one element row per segment) and the values; no memset, no scatter map.
// Dirichlet rows become identity rows and Dirichlet columns zeros, as in the element scatter.
constexpr int GS_WARPS = 4;   // independent warps per block
constexpr int GS_NODES = 31;  // node columns per strip
constexpr int GS_BLOCKS_PER_SM = 8;  // float32: 32 warps per SM, at most 64 registers a thread (float64: half)

// round-to-nearest reciprocals: the correctly rounded 1 / x of either type
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

__device__ __forceinline__ int sym4(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return lo * 4 - lo * (lo - 1) / 2 + (hi - lo);  // row-major upper triangle of a 4 x 4
}

// upper triangle of k int g_a . g_b over one bilinear quad (2 x 2 Gauss points), nodes in
// the mesher's order
template <typename T, bool AFFINE>
__device__ __forceinline__ void quad_stiffness(const T (&x)[4][2], T k, T (&K)[10]) {
#pragma unroll
  for (int u = 0; u < 10; ++u) K[u] = 0;
  // w det J g_a . g_b = dN_a^T M dN_b with M = adj(J) adj(J)^T / det J (Gauss weight 1):
  // per point J, det J and the three entries of M, then three FMAs per pair with the
  // reference derivatives as compile-time constants.  A parallelogram (x0 + x2 = x1 + x3)
  // has one J for all points: then K = M00 C00 + M01 C01 + M11 C11 with the point sums
  // C.. of the derivative products, three FMAs per pair in all.
  const T ex = x[0][0] + x[2][0] - x[1][0] - x[3][0], ey = x[0][1] + x[2][1] - x[1][1] - x[3][1];
  const T scale = fabs(x[2][0] - x[0][0]) + fabs(x[2][1] - x[0][1]) + fabs(x[1][0] - x[3][0]) +
                  fabs(x[1][1] - x[3][1]);
  // AFFINE: every element of the grid is a parallelogram (checked once on the float64
  // coordinates when the grid was recognised)
  const bool affine = AFFINE || fabs(ex) + fabs(ey) <= scale * (sizeof(T) == 4 ? T(1e-6) : T(1e-13));
  if (affine) {
    // J = (1/2) [x1 - x0 | x3 - x0] in the mesher's node order (dN constant in the other
    // variable's direction cancels for a parallelogram)
    const T J00 = T(0.5) * (x[1][0] - x[0][0]), J01 = T(0.5) * (x[3][0] - x[0][0]);
    const T J10 = T(0.5) * (x[1][1] - x[0][1]), J11 = T(0.5) * (x[3][1] - x[0][1]);
    const T rdet = k * rcp_rn(J00 * J11 - J01 * J10);  // the coefficient k folded in
    const T M00 = (J11 * J11 + J01 * J01) * rdet;
    const T M01 = -(J11 * J10 + J01 * J00) * rdet;
    const T M11 = (J10 * J10 + J00 * J00) * rdet;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = a; b < 4; ++b) {
        T c00 = 0, c01 = 0, c11 = 0;  // compile-time sums over the four points
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const T xq = (T)gauss_point(q & 1), yq = (T)gauss_point((q >> 1) & 1);
          const T fa0 = (T(1) + T(node_sign<AGX_QUAD4>(a, 0)) * xq) * T(0.5);
          const T fa1 = (T(1) + T(node_sign<AGX_QUAD4>(a, 1)) * yq) * T(0.5);
          const T fb0 = (T(1) + T(node_sign<AGX_QUAD4>(b, 0)) * xq) * T(0.5);
          const T fb1 = (T(1) + T(node_sign<AGX_QUAD4>(b, 1)) * yq) * T(0.5);
          const T da0 = T(node_sign<AGX_QUAD4>(a, 0)) * T(0.5) * fa1, da1 = T(node_sign<AGX_QUAD4>(a, 1)) * T(0.5) * fa0;
          const T db0 = T(node_sign<AGX_QUAD4>(b, 0)) * T(0.5) * fb1, db1 = T(node_sign<AGX_QUAD4>(b, 1)) * T(0.5) * fb0;
          c00 += da0 * db0;
          c01 += da0 * db1 + da1 * db0;
          c11 += da1 * db1;
        }
        K[sym4(a, b)] = M00 * c00 + M01 * c01 + M11 * c11;
      }
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T dN[4][2];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const T f0 = (T(1) + T(node_sign<AGX_QUAD4>(a, 0)) * (T)gauss_point(q & 1)) * T(0.5);
        const T f1 = (T(1) + T(node_sign<AGX_QUAD4>(a, 1)) * (T)gauss_point((q >> 1) & 1)) * T(0.5);
        dN[a][0] = T(node_sign<AGX_QUAD4>(a, 0)) * T(0.5) * f1;
        dN[a][1] = T(node_sign<AGX_QUAD4>(a, 1)) * T(0.5) * f0;
      }
      T J00 = 0, J01 = 0, J10 = 0, J11 = 0;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        J00 += x[a][0] * dN[a][0];
        J01 += x[a][0] * dN[a][1];
        J10 += x[a][1] * dN[a][0];
        J11 += x[a][1] * dN[a][1];
      }
      const T rdet = rcp_rn(J00 * J11 - J01 * J10);
      const T M00 = (J11 * J11 + J01 * J01) * rdet;
      const T M01 = -(J11 * J10 + J01 * J00) * rdet;
      const T M11 = (J10 * J10 + J00 * J00) * rdet;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = a; b < 4; ++b)
          K[sym4(a, b)] += M00 * (dN[a][0] * dN[b][0]) + M01 * (dN[a][0] * dN[b][1] + dN[a][1] * dN[b][0]) +
                           M11 * (dN[a][1] * dN[b][1]);
    }
#pragma unroll
    for (int u = 0; u < 10; ++u) K[u] *= k;
  }
}

template <int MODEL, typename T, bool AFFINE>
__global__ void __launch_bounds__(GS_WARPS * 32, sizeof(T) == 4 ? GS_BLOCKS_PER_SM : GS_BLOCKS_PER_SM / 2)
grid_tangent_kernel(int nx, int ny, const T* __restrict__ coords, const T* __restrict__ elem_field,
                    const uint8_t* __restrict__ dmask_node, const int32_t* __restrict__ rowptr, T* __restrict__ vals,
                    T* __restrict__ dinv) {
  using V2 = typename std::conditional<std::is_same<T, float>::value, float2, double2>::type;
  using V = typename std::conditional<std::is_same<T, float>::value, float4, double2>::type;
  constexpr int GVEC = 16 / (int)sizeof(T);  // values per 16-byte store
  // a strip's values of one node row plus up to GVEC - 1 words of lead-in, in whole 16-byte chunks
  constexpr int SROW = (GS_NODES * 9 + 2 * GVEC - 2) / GVEC * GVEC;
  __shared__ __align__(16) T stage[GS_WARPS][SROW];
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  // node and element indices fit in 32 bits (agx_set_nodes rejects 2^31 nodes or more)
  const int W = ny + 1, rows = nx + 1;
  const int n_strips = (W + GS_NODES - 1) / GS_NODES;
  // warp gw walks strip gw % n_strips over the node rows of segment gw / n_strips: the rows are
  // split into as many segments as every strip can have (row counts within one of each
  // other), and neighbouring warps take neighbouring strips of the same rows, so that the
  // rows in flight are read and written across their whole width.  One wave of warps.
  const int64_t nw = (int64_t)gridDim.x * GS_WARPS, gw = (int64_t)blockIdx.x * GS_WARPS + wib;
  const int64_t nseg = nw / n_strips;
  const int strip = (int)(gw % n_strips);
  const int64_t seg = gw / n_strips;
  const int64_t ns = max(nseg, (int64_t)1);
  const int i_begin = (int)(rows * seg / ns), i_end = (int)(rows * (seg + 1) / ns);
  if (seg >= nseg || i_begin >= i_end) return;  // whole warps; the kernel has no block-wide barrier
  const int c0 = strip * GS_NODES;           // first node column of the strip (owned by lane 1)
  const int col = c0 + lane - 1;             // this lane's node column and element column
  const bool has_elem = col >= 0 && col < ny;
  const bool owner = lane >= 1 && col <= ny;  // lane owns node (i, col) of every row i
  const bool strip_interior = c0 >= 1 && c0 + GS_NODES - 1 < ny;  // every owned node has both column neighbours
  // Every load is unconditional, at indices clamped into the grid.  A clamped row or column
  // only feeds elements that do not exist (their matrices are zero) and flags of stencil
  // entries outside the grid (never stored), so no load needs a branch.
  const int colc = min(max(col, 0), ny);                 // node column
  const int colx = min(c0 + GS_NODES, ny);               // lane 31: the column right of its node
  const int cole = min(max(col, 0), ny - 1);             // element column
  const int colr = min(max(col + 1, 0), W);              // row pointer of the next node (the row end last)
  const V2* cp = reinterpret_cast<const V2*>(coords);
  T* st = stage[wib];
  auto rowc = [&](int n) { return min(max(n, 0), nx); };

  // per node row n: (x, y) of this lane's node and of the node to its right, and the Dirichlet
  // flags of the left, own and right node as bits 0, 1, 2
  auto right_of = [&](V2 own, V2 ex) {
    V2 r;
    r.x = __shfl_down_sync(FULL, own.x, 1);
    r.y = __shfl_down_sync(FULL, own.y, 1);
    return lane == 31 ? ex : r;
  };
  auto pattern = [&](unsigned own, unsigned ex) {
    const unsigned l = __shfl_up_sync(FULL, own, 1), r = __shfl_down_sync(FULL, own, 1);
    return l | (own << 1) | ((lane == 31 ? ex : r) << 2);
  };
  auto element = [&](int r, V2 b0, V2 b1, V2 t0, V2 t1, T k, T (&K)[10]) {
#pragma unroll
    for (int u = 0; u < 10; ++u) K[u] = 0;
    if (r >= 0 && r < nx && has_elem) {
      const T x[4][2] = {{b0.x, b0.y}, {b1.x, b1.y}, {t1.x, t1.y}, {t0.x, t0.y}};
      quad_stiffness<T, AFFINE>(x, k, K);
    }
  };
  auto coefficient = [&](int r) {
    if constexpr (MODEL == AGX_MODEL_HEAT_POTENTIAL)
      if (elem_field) return elem_field[min(max(r, 0), nx - 1) * ny + cole];
    return T(1);
  };

  // the element row above the segment (i_begin - 1), the state entering row i_begin and,
  // already in flight while that element is integrated, the loads one row ahead: node row
  // i + 1 (the top of element row i), element row i's coefficients, node row i's row pointers
  T Kp[10];
  V2 bottom, bottom_r;
  unsigned pat_up, pat_mid;
  int rn = rowc(i_begin - 1) * W;
  const V2 ao = cp[rn + colc], ax = cp[rn + colx];
  const unsigned fa = dmask_node[rn + colc] & 1u, fax = dmask_node[rn + colx] & 1u;
  rn = rowc(i_begin) * W;
  const V2 bo = cp[rn + colc], bx = cp[rn + colx];
  const unsigned fb = dmask_node[rn + colc] & 1u, fbx = dmask_node[rn + colx] & 1u;
  const T ka = coefficient(i_begin - 1);
  rn = rowc(i_begin + 1) * W;
  V2 nto = cp[rn + colc], ntx = cp[rn + colx];
  unsigned nfo = dmask_node[rn + colc], nfx = dmask_node[rn + colx];
  T nk = coefficient(i_begin);
  int32_t nrp = rowptr[i_begin * W + colr];
  pat_up = pattern(fa, fax);
  pat_mid = pattern(fb, fbx);
  bottom = bo;
  bottom_r = right_of(bo, bx);
  element(i_begin - 1, ao, right_of(ao, ax), bo, bottom_r, ka, Kp);

  // two rows per trip: the element-row registers alternate without copies
#pragma unroll 2
  for (int i = i_begin; i < i_end; ++i) {
    const V2 top = nto, topx = ntx;
    const unsigned tfo = nfo & 1u, tfx = nfx & 1u;
    const T kc = nk;
    const int32_t rpn = nrp;
    rn = rowc(i + 2) * W;  // the next row's loads, in flight while this row is computed
    nto = cp[rn + colc];
    ntx = cp[rn + colx];
    nfo = dmask_node[rn + colc];
    nfx = dmask_node[rn + colx];
    nk = coefficient(i + 1);
    nrp = rowptr[min(i + 1, nx) * W + colr];

    const V2 top_r = right_of(top, topx);
    const unsigned pat_dn = pattern(tfo, tfx);
    T Kc[10];
    element(i, bottom, bottom_r, top, top_r, kc, Kc);
    // this lane's elements' share of the row of its own node (i, col) and of the node to its
    // right (i, col + 1): entries (row offset, column offset) of the 3 x 3 stencil
    const T o_m0 = Kp[sym4(3, 0)], o_m1 = Kp[sym4(3, 1)];
    const T o_01 = Kp[sym4(3, 2)] + Kc[sym4(0, 1)], o_00 = Kp[sym4(3, 3)] + Kc[sym4(0, 0)];
    const T o_p1 = Kc[sym4(0, 2)], o_p0 = Kc[sym4(0, 3)];
    const T r_mm = Kp[sym4(2, 0)], r_m0 = Kp[sym4(2, 1)];
    const T r_00 = Kp[sym4(2, 2)] + Kc[sym4(1, 1)], r_0m = Kp[sym4(2, 3)] + Kc[sym4(1, 0)];
    const T r_p0 = Kc[sym4(1, 2)], r_pm = Kc[sym4(1, 3)];
    T v[9];  // (di + 1) * 3 + (dj + 1)
    v[0] = __shfl_up_sync(FULL, r_mm, 1);
    v[1] = __shfl_up_sync(FULL, r_m0, 1) + o_m0;
    v[2] = o_m1;
    v[3] = __shfl_up_sync(FULL, r_0m, 1);
    v[4] = __shfl_up_sync(FULL, r_00, 1) + o_00;
    v[5] = o_01;
    v[6] = __shfl_up_sync(FULL, r_pm, 1);
    v[7] = __shfl_up_sync(FULL, r_p0, 1) + o_p0;
    v[8] = o_p1;
    if (__any_sync(FULL, (pat_up | pat_mid | pat_dn) != 0u)) {
      if (pat_mid & 2u) {  // a prescribed node: identity row
#pragma unroll
        for (int u = 0; u < 9; ++u) v[u] = T(0);
        v[4] = T(1);
      } else {  // prescribed columns are deleted
#pragma unroll
        for (int dj = 0; dj < 3; ++dj) {
          if ((pat_up >> dj) & 1u) v[dj] = T(0);
          if ((pat_mid >> dj) & 1u) v[3 + dj] = T(0);
          if ((pat_dn >> dj) & 1u) v[6 + dj] = T(0);
        }
      }
    }
    // the Jacobi inverse diagonal of the row (the inverse_diagonal pass, fused); the
    // round-to-nearest reciprocal is the correctly rounded 1 / x
    if (owner) dinv[i * W + col] = v[4] != T(0) ? rcp_rn(v[4]) : T(0);
    // the strip's rows are consecutive nodes: one contiguous range of values [base, end),
    // staged so that global value base + u sits at stage word shift + u and 16-byte chunks
    // line up.  Lane l's row starts where lane l - 1's next-node row pointer points.
    const int32_t base = __shfl_sync(FULL, rpn, 0), end = __shfl_sync(FULL, rpn, 31);
    const int32_t rp = __shfl_up_sync(FULL, rpn, 1);
    const int shift = base & (GVEC - 1);
    if (owner) {
      T* sr = st + shift + (rp - base);
      if (strip_interior && i >= 1 && i < nx) {
#pragma unroll
        for (int u = 0; u < 9; ++u) sr[u] = v[u];
      } else {
        int idx = 0;
#pragma unroll
        for (int di = -1; di <= 1; ++di)
#pragma unroll
          for (int dj = -1; dj <= 1; ++dj)
            if (i + di >= 0 && i + di <= nx && col + dj >= 0 && col + dj <= ny)
              sr[idx++] = v[(di + 1) * 3 + (dj + 1)];
      }
    }
    __syncwarp();
    {
      const int end_w = shift + (end - base);
      const int first_full = (shift + GVEC - 1) / GVEC, last_full = end_w / GVEC;
      V* dst = reinterpret_cast<V*>(vals + (base - shift));
      const V* src = reinterpret_cast<const V*>(st);
      for (int c = first_full + lane; c < last_full; c += 32) dst[c] = src[c];
      // the partial first and last chunks, word by word (at most GVEC - 1 words each)
      const int hw = shift + lane, head_end = min(first_full * GVEC, end_w);
      if (lane < GVEC - 1 && hw < head_end) vals[base - shift + hw] = st[hw];
      const int tw = max(last_full, first_full) * GVEC + (lane - 16);
      if (lane >= 16 && lane < 16 + GVEC - 1 && tw < end_w) vals[base - shift + tw] = st[tw];
    }
    __syncwarp();  // the stage is rewritten by the next row
#pragma unroll
    for (int u = 0; u < 10; ++u) Kp[u] = Kc[u];
    bottom = top;
    bottom_r = top_r;
    pat_up = pat_mid;
    pat_mid = pat_dn;
  }
}

// ---- float64 neo-Hooke residual, one Gauss point per lane ---------------------------------
// With NQ = NEN Gauss points (2 per direction on Q1 quads and bricks), lane l of an element's
// lane group is node l for the DOFs and the scatter and Gauss point l for the constitutive
// law: it forms F = I + sum_b u_b (x) g_b(q_l) from the float64 geometry cache and the other
// lanes' DOFs (shuffles), evaluates P = mu F + c F^-T once (instead of once per node), and
// after an exchange of w det J P through shared memory forms R_l,i = sum_q (w det J P_q)_iJ
// g_l,J(q).  Same quantities as element_kernel<NEO_HOOKE, double, residual only>, the
// constitutive work divided by NEN.
template <int ET>
__global__ void __launch_bounds__(AGX_BLOCK)
neo_hooke_residual_qp(int64_t n_elem, const int32_t* __restrict__ conn, const double* __restrict__ dofs,
                      const double* __restrict__ geo, ModelParams mp, double* __restrict__ R) {
  constexpr int NEN = ElemTraits<ET>::NEN, NQ = NEN;
  constexpr int SDIM = space_dim<ET>();
  __shared__ double Psh[AGX_BLOCK / 32][32][SDIM * SDIM];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int l = lane % NEN, gbase = lane - l;
  const double E = mp.p[0], nu = mp.p[1];
  const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = E / (2.0 * (1.0 + nu));
  const int64_t total = ((n_elem * NEN + 31) / 32) * 32;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e_raw = L / NEN;
    const bool valid = e_raw < n_elem;
    const int64_t e = valid ? e_raw : n_elem - 1;
    const int node = conn[e * NEN + l];
    double ul[SDIM];
#pragma unroll
    for (int c = 0; c < SDIM; ++c) ul[c] = dofs[(int64_t)node * SDIM + c];
    // displacement gradient H = F - I at Gauss point l
    double F[SDIM][SDIM];
#pragma unroll
    for (int i = 0; i < SDIM; ++i)
#pragma unroll
      for (int j = 0; j < SDIM; ++j) F[i][j] = 0.0;
    const double* gq = geo + ((e * NQ + l) * NEN) * (SDIM + 1);
#pragma unroll
    for (int b = 0; b < NEN; ++b) {
      double ub[SDIM], g[SDIM];
#pragma unroll
      for (int c = 0; c < SDIM; ++c) ub[c] = __shfl_sync(0xffffffffu, ul[c], gbase + b);
#pragma unroll
      for (int d = 0; d < SDIM; ++d) g[d] = gq[b * (SDIM + 1) + d];
#pragma unroll
      for (int i = 0; i < SDIM; ++i)
#pragma unroll
        for (int j = 0; j < SDIM; ++j) F[i][j] += ub[i] * g[j];
    }
    const double wdet = gq[SDIM];  // w det J at this point (stored with every node)
    double Fi[SDIM][SDIM], P[SDIM][SDIM], J;
    neo_hooke_stress<double, SDIM>(F, lam, mu, P, Fi, J);
    __syncwarp();
#pragma unroll
    for (int i = 0; i < SDIM; ++i)
#pragma unroll
      for (int j = 0; j < SDIM; ++j) Psh[warp][lane][i * SDIM + j] = wdet * P[i][j];
    __syncwarp();
    // R_l = sum over points q of (w det J P_q) g_l(q)
    double Rl[SDIM];
#pragma unroll
    for (int i = 0; i < SDIM; ++i) Rl[i] = 0.0;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const double* gl = geo + ((e * NQ + q) * NEN + l) * (SDIM + 1);
      double g[SDIM];
#pragma unroll
      for (int d = 0; d < SDIM; ++d) g[d] = gl[d];
#pragma unroll
      for (int i = 0; i < SDIM; ++i)
#pragma unroll
        for (int j = 0; j < SDIM; ++j) Rl[i] += Psh[warp][gbase + q][i * SDIM + j] * g[j];
    }
    if (valid) {
#pragma unroll
      for (int i = 0; i < SDIM; ++i) atomicAdd(R + (int64_t)node * SDIM + i, Rl[i]);
    }
  }
}

// prescribed diagonal entries of the (zeroed) value array set to one
template <typename T>
__global__ void set_dirichlet_diag(int64_t n_dir, const int32_t* __restrict__ dir_dofs,
                                   const int32_t* __restrict__ diagpos, int ndof, int64_t nnzb,
                                   T* __restrict__ vals) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n_dir; k += (int64_t)gridDim.x * blockDim.x) {
    const int d = dir_dofs[k];
    const int p = d / ndof, c = d - p * ndof;
    vals[(int64_t)(c * ndof + c) * nnzb + diagpos[p]] = T(1);
  }
}

// inverse diagonal for Jacobi
template <typename T>
__global__ void inverse_diagonal(int64_t n_dofs, int ndof, int64_t nnzb, const int32_t* __restrict__ diagpos,
                                 const T* __restrict__ vals, T* __restrict__ dinv) {
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n_dofs; d += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = d / ndof;
    const int c = (int)(d - p * ndof);
    const T v = vals[(int64_t)(c * ndof + c) * nnzb + diagpos[p]];
    dinv[d] = v != T(0) ? T(1) / v : T(0);
  }
}

// diagonal of the assembled tangent in float64 (assemble_tangent_diagonal)
template <typename T>
__global__ void tangent_diagonal(int64_t n_dofs, int ndof, int64_t nnzb, const int32_t* __restrict__ diagpos,
                                 const T* __restrict__ vals, double* __restrict__ diag) {
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n_dofs; d += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = d / ndof;
    const int c = (int)(d - p * ndof);
    diag[d] = (double)vals[(int64_t)(c * ndof + c) * nnzb + diagpos[p]];
  }
}

// the coordinates and element field in a pass's arithmetic type (float32 copies made at set-up)
template <typename T>
const T* coords_of(const agx_context* ctx) {
  if constexpr (std::is_same<T, double>::value) return ctx->d_coords;
  else return ctx->d_coords32;
}
template <typename T>
const T* elem_field_of(const agx_element_set& s) {
  if constexpr (std::is_same<T, double>::value) return s.d_elem_field;
  else return s.d_elem_field32;
}

template <int ET, int MODEL, typename T, bool DO_R, bool DO_K>
void launch_element(agx_context* ctx, agx_element_set& s, const double* dofs, double* R, T* vals,
                    double* geo_out = nullptr) {
  // the float64 passes read the geometry cache once it exists
  const double* geo = (std::is_same<T, double>::value && geo_out == nullptr) ? s.d_geo : nullptr;
  ModelParams mp;
  for (int i = 0; i < AGX_MAX_PARAMS; ++i) mp.p[i] = s.params[i];
  const int64_t lanes = s.n_elem * ElemTraits<ET>::GROUP;
  const int grid = agx_grid(ctx, lanes, 8);
  QuadTable qt;
  qt.n = s.nqp;
  for (int q = 0; q < AGX_MAX_QPOINTS; ++q) {
    for (int d = 0; d < 3; ++d) qt.x[q][d] = s.qp[q][d];
    qt.w[q] = s.qw[q];
  }
  if constexpr (ET == AGX_HEX27 && MODEL == AGX_MODEL_NEO_HOOKE && DO_K) {
    // 27 nodes x 3 DOFs: the tangent row in column chunks (9 nodes in float32, 5 in float64), the
    // residual with the first chunk
    constexpr int CBk = std::is_same<T, double>::value ? 5 : 9;
    for (int b0 = 0; b0 < 27; b0 += CBk) {
      if (b0 == 0)
        element_kernel<ET, MODEL, T, DO_R, true, CBk><<<grid, AGX_BLOCK, 0, ctx->stream>>>(
            s.n_elem, s.d_conn, s.d_epos, coords_of<T>(ctx), dofs, elem_field_of<T>(s), s.d_node_field,
            ctx->d_dmask_node, mp, R, vals, ctx->nnzb, geo, geo_out, s.ngauss, qt, b0);
      else
        element_kernel<ET, MODEL, T, false, true, CBk><<<grid, AGX_BLOCK, 0, ctx->stream>>>(
            s.n_elem, s.d_conn, s.d_epos, coords_of<T>(ctx), dofs, elem_field_of<T>(s), s.d_node_field,
            ctx->d_dmask_node, mp, nullptr, vals, ctx->nnzb, geo, nullptr, s.ngauss, qt, b0);
      ctx->n_launches += 1;
    }
  } else {
    element_kernel<ET, MODEL, T, DO_R, DO_K><<<grid, AGX_BLOCK, 0, ctx->stream>>>(
        s.n_elem, s.d_conn, s.d_epos, coords_of<T>(ctx), dofs, elem_field_of<T>(s), s.d_node_field,
        ctx->d_dmask_node, mp, R, vals, ctx->nnzb, geo, geo_out, s.ngauss, qt);
    ctx->n_launches += 1;
  }
}

// ---- float64 residual of the heat potential on a uniform structured quad grid ---------------
// Every element is the same parallelogram, so its 2 x 2 Gauss-point stiffness per unit
// coefficient is one 4 x 4 matrix K0 = M00 C00 + M01 C01 + M11 C11 (C.. the point sums of the
// reference derivative products, M from the constant Jacobian, both as quad_stiffness forms
// them) and every element's load vector is the source times det J (the four shape functions
// sum to 1 at each point).  One lane per node adds the four adjacent elements' rows:
// R_p = sum_e k_e (K0 T_e)_a - f det J, with a the node's place in element e -- one write per
// node, no atomics, no geometry cache (the element kernel reads ~380 bytes of cached
// gradients per element).
__global__ void __launch_bounds__(AGX_BLOCK)
grid_heat_residual(int nx, int ny, const double* __restrict__ kfield, double src, const double* __restrict__ T,
                   double M00, double M01, double M11, double det, double* __restrict__ R) {
  double K0[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      double c00 = 0, c01 = 0, c11 = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double xq = gauss_point(q & 1), yq = gauss_point((q >> 1) & 1);
        const double fa0 = (1.0 + node_sign<AGX_QUAD4>(a, 0) * xq) * 0.5;
        const double fa1 = (1.0 + node_sign<AGX_QUAD4>(a, 1) * yq) * 0.5;
        const double fb0 = (1.0 + node_sign<AGX_QUAD4>(b, 0) * xq) * 0.5;
        const double fb1 = (1.0 + node_sign<AGX_QUAD4>(b, 1) * yq) * 0.5;
        const double da0 = node_sign<AGX_QUAD4>(a, 0) * 0.5 * fa1, da1 = node_sign<AGX_QUAD4>(a, 1) * 0.5 * fa0;
        const double db0 = node_sign<AGX_QUAD4>(b, 0) * 0.5 * fb1, db1 = node_sign<AGX_QUAD4>(b, 1) * 0.5 * fb0;
        c00 += da0 * db0;
        c01 += da0 * db1 + da1 * db0;
        c11 += da1 * db1;
      }
      K0[a][b] = M00 * c00 + M01 * c01 + M11 * c11;
    }
  const int W = ny + 1;
  const int64_t n = (int64_t)(nx + 1) * W;
  const double load = src * det;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p / W), j = (int)(p - (int64_t)i * W);
    double acc = 0.0;
    // the element (ei, ej) = (i - di, j - dj) holds node p at local (di, dj): mesher order
    // (0, 0) -> 0, (0, 1) -> 1, (1, 1) -> 2, (1, 0) -> 3
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
      for (int dj = 0; dj < 2; ++dj) {
        const int ei = i - di, ej = j - dj;
        if (ei < 0 || ei >= nx || ej < 0 || ej >= ny) continue;
        const int a = di == 0 ? (dj == 0 ? 0 : 1) : (dj == 0 ? 3 : 2);
        const int64_t n0 = (int64_t)ei * W + ej;
        const double t0 = T[n0], t1 = T[n0 + 1], t2 = T[n0 + W + 1], t3 = T[n0 + W];
        const double ke = kfield ? kfield[(int64_t)ei * ny + ej] : 1.0;
        acc += ke * (K0[a][0] * t0 + K0[a][1] * t1 + K0[a][2] * t2 + K0[a][3] * t3) - load;
      }
    R[p] += acc;
  }
}

// dispatch on (element type, model) for one pass kind// dispatch on (element type, model) for one pass kind
template <typename T, bool DO_R, bool DO_K>
int dispatch(agx_context* ctx, agx_element_set& s, const double* dofs, double* R, T* vals) {
  if constexpr (std::is_same<T, double>::value && DO_R && !DO_K) {
    if (agx_brick_heat_be(ctx, s)) {
      agx_launch_brick_residual(ctx, s, dofs, R);
      return AGX_OK;
    }
    if (s.model == AGX_MODEL_HEAT_POTENTIAL && s.elem_type == AGX_QUAD4 && s.grid_nx > 0 && s.grid_uniform &&
        s.ngauss == 2 && ctx->ndof == 1) {
      grid_heat_residual<<<agx_grid(ctx, (int64_t)(s.grid_nx + 1) * (s.grid_ny + 1)), AGX_BLOCK, 0, ctx->stream>>>(
          s.grid_nx, s.grid_ny, s.d_elem_field, s.params[0], dofs, s.grid_m[0], s.grid_m[1], s.grid_m[2], s.grid_m[3],
          R);
      ctx->n_launches += 1;
      return AGX_OK;
    }
    if (s.model == AGX_MODEL_NEO_HOOKE && s.d_geo && s.ngauss == 2 &&
        (s.elem_type == AGX_HEX8 || s.elem_type == AGX_QUAD4)) {
      ModelParams mp;
      for (int i = 0; i < AGX_MAX_PARAMS; ++i) mp.p[i] = s.params[i];
      const int64_t lanes = s.n_elem * s.nen;
      const int grid = agx_grid(ctx, lanes, 8);
      if (s.elem_type == AGX_HEX8)
        neo_hooke_residual_qp<AGX_HEX8><<<grid, AGX_BLOCK, 0, ctx->stream>>>(s.n_elem, s.d_conn, dofs, s.d_geo, mp, R);
      else
        neo_hooke_residual_qp<AGX_QUAD4><<<grid, AGX_BLOCK, 0, ctx->stream>>>(s.n_elem, s.d_conn, dofs, s.d_geo, mp, R);
      ctx->n_launches += 1;
      return AGX_OK;
    }
  }
#define AGX_CASE(ETV, MV)                                                  \
  if (s.elem_type == ETV && s.model == MV) {                               \
    launch_element<ETV, MV, T, DO_R, DO_K>(ctx, s, dofs, R, vals);         \
    return AGX_OK;                                                         \
  }
  AGX_CASE(AGX_QUAD4, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_QUAD4, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_QUAD4, AGX_MODEL_NEO_HOOKE)
  AGX_CASE(AGX_QUAD4, AGX_MODEL_HEAT_BE)
  AGX_CASE(AGX_HEX8, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_HEX8, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_HEX8, AGX_MODEL_NEO_HOOKE)
  AGX_CASE(AGX_HEX8, AGX_MODEL_HEAT_BE)
  AGX_CASE(AGX_LINE2, AGX_MODEL_NEUMANN)
  AGX_CASE(AGX_QUAD9, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_QUAD9, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_QUAD9, AGX_MODEL_NEO_HOOKE)
  AGX_CASE(AGX_LINE3, AGX_MODEL_NEUMANN)
  AGX_CASE(AGX_TRI3, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_TRI3, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_TRI3, AGX_MODEL_NEO_HOOKE)
  AGX_CASE(AGX_TRI6, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_TRI6, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_TRI6, AGX_MODEL_NEO_HOOKE)
  AGX_CASE(AGX_TET4, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_TET4, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_TET4, AGX_MODEL_NEO_HOOKE)
  AGX_CASE(AGX_TET10, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_TET10, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_TET10, AGX_MODEL_NEO_HOOKE)
  AGX_CASE(AGX_HEX27, AGX_MODEL_POISSON_SINCOS)
  AGX_CASE(AGX_HEX27, AGX_MODEL_HEAT_POTENTIAL)
  AGX_CASE(AGX_HEX27, AGX_MODEL_NEO_HOOKE)
#undef AGX_CASE
  return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "element type %d with model %d is not supported", s.elem_type, s.model);
}

// one-time float64 geometry pass of a domain set: fills s.d_geo
int build_geometry(agx_context* ctx, agx_element_set& s) {
  if (s.elem_type == AGX_LINE2 || s.elem_type == AGX_LINE3 || s.d_geo) return AGX_OK;
  // simplices and 27-node bricks keep no cache: their geometry is recomputed per pass
  if (s.elem_type == AGX_TRI3 || s.elem_type == AGX_TRI6 || s.elem_type == AGX_TET4 || s.elem_type == AGX_TET10 ||
      s.elem_type == AGX_HEX27)
    return AGX_OK;
  const int sd = s.elem_type == AGX_HEX8 ? 3 : 2;
  const int nq = sd == 3 ? s.ngauss * s.ngauss * s.ngauss : s.ngauss * s.ngauss;
  const size_t bytes = sizeof(double) * (size_t)s.n_elem * nq * s.nen * (sd + 1);
  if (bytes > ctx->geo_cache_limit) return AGX_OK;  // too large: the passes recompute the geometry
  AGX_CUDA(ctx, cudaMalloc((void**)&s.d_geo, bytes));
  // the geometry does not depend on the model: one scalar-model pass serves every model
  if (s.elem_type == AGX_HEX8)
    launch_element<AGX_HEX8, AGX_MODEL_HEAT_POTENTIAL, double, false, false>(ctx, s, nullptr, nullptr, nullptr,
                                                                             s.d_geo);
  else if (s.elem_type == AGX_QUAD9)
    launch_element<AGX_QUAD9, AGX_MODEL_HEAT_POTENTIAL, double, false, false>(ctx, s, nullptr, nullptr, nullptr,
                                                                              s.d_geo);
  else
    launch_element<AGX_QUAD4, AGX_MODEL_HEAT_POTENTIAL, double, false, false>(ctx, s, nullptr, nullptr, nullptr,
                                                                              s.d_geo);
  AGX_CHECK_LAUNCH(ctx);
  return AGX_OK;
}

}  // namespace

// the set whose tangent the structured row kernel writes on its own, or null
static agx_element_set* grid_tangent_set(agx_context* ctx) {
  agx_element_set* hit = nullptr;
  int with_k = 0;
  for (auto& s : ctx->sets) {
    if (s.model == AGX_MODEL_NEUMANN) continue;  // no tangent contribution
    ++with_k;
    if (s.grid_nx > 0 && s.ngauss == 2 && ctx->ndof == 1 &&
        (s.model == AGX_MODEL_HEAT_POTENTIAL || s.model == AGX_MODEL_POISSON_SINCOS))
      hit = &s;
  }
  return with_k == 1 ? hit : nullptr;
}

// the uniform brick set whose float32 tangent the brick row kernel writes on its own, or null
static agx_element_set* brick_tangent_set(agx_context* ctx) {
  agx_element_set* hit = nullptr;
  int with_k = 0;
  for (auto& s : ctx->sets) {
    if (s.model == AGX_MODEL_NEUMANN) continue;
    ++with_k;
    if (agx_brick_heat_be(ctx, s)) hit = &s;
  }
  return with_k == 1 ? hit : nullptr;
}

template <int MODEL, typename T, bool AFFINE>
static void launch_grid_tangent_as(agx_context* ctx, agx_element_set& s, T* vals, T* dinv) {
  // one wave: the resident blocks of every SM (occupancy calculator), never more warps than
  // (strip, node row) pairs and never fewer than strips (one segment of rows each)
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_tangent_kernel<MODEL, T, AFFINE>, GS_WARPS * 32, 0);
    per_sm = std::max(per_sm, 1);
  }
  const int64_t strips = (s.grid_ny + 1 + GS_NODES - 1) / GS_NODES, rows = (int64_t)s.grid_nx + 1;
  const int64_t warps = std::max<int64_t>(strips, std::min<int64_t>((int64_t)ctx->sm_count * per_sm * GS_WARPS, rows * strips));
  const unsigned grid = (unsigned)((warps + GS_WARPS - 1) / GS_WARPS);
  grid_tangent_kernel<MODEL, T, AFFINE><<<grid, GS_WARPS * 32, 0, ctx->stream>>>(
      s.grid_nx, s.grid_ny, coords_of<T>(ctx), elem_field_of<T>(s), ctx->d_dmask_node, ctx->d_rowptr, vals, dinv);
  ctx->n_launches += 1;
}

template <typename T>
static void launch_grid_tangent(agx_context* ctx, agx_element_set& s, T* vals, T* dinv) {
  if (s.model == AGX_MODEL_HEAT_POTENTIAL) {
    if (s.grid_affine) launch_grid_tangent_as<AGX_MODEL_HEAT_POTENTIAL, T, true>(ctx, s, vals, dinv);
    else launch_grid_tangent_as<AGX_MODEL_HEAT_POTENTIAL, T, false>(ctx, s, vals, dinv);
  } else {
    if (s.grid_affine) launch_grid_tangent_as<AGX_MODEL_POISSON_SINCOS, T, true>(ctx, s, vals, dinv);
    else launch_grid_tangent_as<AGX_MODEL_POISSON_SINCOS, T, false>(ctx, s, vals, dinv);
  }
}

void agx_launch_diagonal(agx_context* ctx, int dtype, double* diag) {
  const int g = agx_grid(ctx, ctx->n_dofs);
  if (dtype == AGX_F64)
    tangent_diagonal<double><<<g, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, ctx->ndof, ctx->nnzb, ctx->d_diagpos,
                                                               ctx->d_vals64, diag);
  else
    tangent_diagonal<float><<<g, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, ctx->ndof, ctx->nnzb, ctx->d_diagpos,
                                                              ctx->d_vals32, diag);
  ctx->n_launches += 1;
}

int agx_assemble_impl(agx_context* ctx, const double* dofs, double* residual, int tangent_dtype) {
  const int bs = ctx->ndof * ctx->ndof;
  for (auto& s : ctx->sets)
    if ((s.elem_type == AGX_TRI3 || s.elem_type == AGX_TRI6 || s.elem_type == AGX_TET4 || s.elem_type == AGX_TET10) &&
        s.nqp < 1)
      return agx_fail(ctx, AGX_ERR_STATE, "simplex set without integration points (agx_set_quadrature_points)");
  agx_element_set* gset = tangent_dtype >= 0 ? grid_tangent_set(ctx) : nullptr;
  // the uniform brick grid's row kernel (float32 tangents; float64 ones keep the element pass)
  agx_element_set* bset = (!gset && tangent_dtype == AGX_F32) ? brick_tangent_set(ctx) : nullptr;
  if (residual || tangent_dtype == AGX_F64)
    for (auto& s : ctx->sets)
      if (int rc = build_geometry(ctx, s)) return rc;
  if (residual) AGX_CUDA(ctx, cudaMemsetAsync(residual, 0, sizeof(double) * ctx->n_dofs, ctx->stream));
  if (gset || bset) {
    // every entry of every row is written by the row kernel: no zeroing, no diagonal pass
  } else if (tangent_dtype == AGX_F64) {
    AGX_CUDA(ctx, cudaMemsetAsync(ctx->d_vals64, 0, sizeof(double) * ctx->nnzb * bs, ctx->stream));
    if (ctx->n_dir > 0)
      set_dirichlet_diag<double><<<agx_grid(ctx, ctx->n_dir), AGX_BLOCK, 0, ctx->stream>>>(
          ctx->n_dir, ctx->d_dir_dofs, ctx->d_diagpos, ctx->ndof, ctx->nnzb, ctx->d_vals64);
  } else if (tangent_dtype == AGX_F32) {
    AGX_CUDA(ctx, cudaMemsetAsync(ctx->d_vals32, 0, sizeof(float) * ctx->nnzb * bs, ctx->stream));
    if (ctx->n_dir > 0)
      set_dirichlet_diag<float><<<agx_grid(ctx, ctx->n_dir), AGX_BLOCK, 0, ctx->stream>>>(
          ctx->n_dir, ctx->d_dir_dofs, ctx->d_diagpos, ctx->ndof, ctx->nnzb, ctx->d_vals32);
  }
  for (auto& s : ctx->sets) {
    int rc = AGX_OK;
    if (gset == &s) {
      {
        agx_prof_scope ps(ctx, AGX_PROF_TANGENT);
        if (tangent_dtype == AGX_F64)
          launch_grid_tangent<double>(ctx, s, ctx->d_vals64, ctx->d_dinv64);
        else
          launch_grid_tangent<float>(ctx, s, ctx->d_vals32, ctx->d_dinv32);
      }
      if (residual) {
        agx_prof_scope ps(ctx, AGX_PROF_RESIDUAL);
        rc = dispatch<double, true, false>(ctx, s, dofs, residual, (double*)nullptr);
      }
    } else if (bset == &s) {
      {
        agx_prof_scope ps(ctx, AGX_PROF_TANGENT);
        agx_launch_brick_tangent(ctx, s, dofs, ctx->d_vals32, ctx->d_dinv32);
      }
      if (residual) {
        agx_prof_scope ps(ctx, AGX_PROF_RESIDUAL);
        rc = dispatch<double, true, false>(ctx, s, dofs, residual, (double*)nullptr);
      }
    } else if ((gset || bset) && s.model != AGX_MODEL_NEUMANN) {
      rc = AGX_ERR_STATE;  // unreachable: the row kernel serves the only set with a tangent
    } else if (tangent_dtype == AGX_F64) {
      agx_prof_scope ps(ctx, AGX_PROF_TANGENT);
      rc = residual ? dispatch<double, true, true>(ctx, s, dofs, residual, ctx->d_vals64)
                    : dispatch<double, false, true>(ctx, s, dofs, nullptr, ctx->d_vals64);
    } else if (tangent_dtype == AGX_F32) {
      // float32 tangent pass; the float64 residual is a separate float64 pass
      {
        agx_prof_scope ps(ctx, AGX_PROF_TANGENT);
        rc = dispatch<float, false, true>(ctx, s, dofs, nullptr, ctx->d_vals32);
      }
      if (rc == AGX_OK && residual) {
        agx_prof_scope ps(ctx, AGX_PROF_RESIDUAL);
        rc = dispatch<double, true, false>(ctx, s, dofs, residual, (double*)nullptr);
      }
    } else if (residual) {
      agx_prof_scope ps(ctx, AGX_PROF_RESIDUAL);
      rc = dispatch<double, true, false>(ctx, s, dofs, residual, (double*)nullptr);
    }
    if (rc != AGX_OK) return rc;
    AGX_CHECK_LAUNCH(ctx);
  }
  if (tangent_dtype >= 0 && !gset && !bset) ctx->n_launches += (ctx->n_dir > 0 ? 2 : 1);  // Dirichlet diagonal + inverse diagonal
  if (gset || bset) {
    ctx->tangent_valid = tangent_dtype;  // the row kernel wrote the inverse diagonal
  } else if (tangent_dtype == AGX_F64) {
    inverse_diagonal<double><<<agx_grid(ctx, ctx->n_dofs), AGX_BLOCK, 0, ctx->stream>>>(
        ctx->n_dofs, ctx->ndof, ctx->nnzb, ctx->d_diagpos, ctx->d_vals64, ctx->d_dinv64);
    ctx->tangent_valid = AGX_F64;
  } else if (tangent_dtype == AGX_F32) {
    inverse_diagonal<float><<<agx_grid(ctx, ctx->n_dofs), AGX_BLOCK, 0, ctx->stream>>>(
        ctx->n_dofs, ctx->ndof, ctx->nnzb, ctx->d_diagpos, ctx->d_vals32, ctx->d_dinv32);
    ctx->tangent_valid = AGX_F32;
  }
  if (tangent_dtype >= 0) ctx->tangent_gen += 1;
  AGX_CHECK_LAUNCH(ctx);
  return AGX_OK;
}
