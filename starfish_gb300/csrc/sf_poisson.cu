// sf_poisson.cu -- nonlinear Poisson solve with Boltzmann electrons, electric field.
//
// The reference (pic/PoissonSolver.java:110-252, core/solver/Solver.java:293-387,
// LinearSolverGS.java:74-152) assembles an FVM matrix A (5-point on a uniform XY mesh,
// identity rows on Dirichlet nodes, one-sided gradient rows on open mesh faces), then
// runs Newton on  F(x) = A x - b0 - (e n0/eps) exp((x - phi0)/kTe)  with J = A - diag(P),
// solving each J y = F by SOR.
//
// Here the same operator is applied in closed form (no matrix is stored) and the solve
// is built for GB300, whose FP64 rate is a small fraction of its FP32 rate:
//   * outer loop in FP64: residual F, its norm and the update x -= y -- the quantities
//     whose precision decides the converged potential (iterative refinement);
//   * inner correction in FP32: flexible conjugate gradients preconditioned by one
//     geometric multigrid V(2,2)-cycle (red-black Gauss-Seidel, full weighting, bilinear
//     prolongation).  A plain V-cycle converges poorly here because the coarse grids
//     see the embedded electrode only approximately; CG removes those few slow modes.
//     The operator is made symmetric by scaling the open-face (one-sided gradient) rows
//     by 1/h, which leaves its solution unchanged.
// The coarse end of the hierarchy runs inside one CTA out of shared memory, so a V-cycle
// is a handful of launches: from COARSE_NODES nodes down for one mesh, and from
// COARSE_NODES_BATCH down in the batched solve, where many instances' single-CTA cycles
// run side by side.  Every level does the same arithmetic in the CTA as in the global
// level kernels, so the split does not change the result.  All inner scalars stay on the
// device; the host reads one FP64 residual norm per Newton step.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "sf_internal.h"

using namespace sf;

namespace {

// node classes of the closed-form operator
enum : uint8_t { NC_INTERIOR = 0, NC_FIXED = 1, NC_NLEFT = 2, NC_NRIGHT = 3, NC_NBOTTOM = 4, NC_NTOP = 5 };

constexpr int COARSE_NODES = 2200;        // one mesh: a level this small and all below in one CTA
constexpr int COARSE_NODES_BATCH = 8600;  // the same for the batched solve
constexpr size_t COARSE_SMEM_MAX = 220 * 1024;  // dynamic shared memory bound of the coarse V-cycle
constexpr int MAX_LEVELS = 16;

struct LevelView {
  int ni, nj;
  float cx, cy;  // 1/dx^2, 1/dy^2
  float* y;
  float* r;
  float* P;
  float* t;  // residual scratch of the batched global-sweep levels
  const uint8_t* type;
};

// Axisymmetric meshes (RZ: radius along i, ZR: along j): the inner FP32 system is the
// reference's Jacobian with every row multiplied by a radius, which makes it symmetric:
// interior rows by 2 pi r (the node's radius; Ax is the cylindrical Laplacian / 2 pi),
// open-face rows by the radius of the face that joins them to the interior.
struct AxiView {
  int axi;       // 1 = RZ, 2 = ZR
  float r0, dr;  // radius of the first node column (RZ) / row (ZR), and the spacing
};

struct CoarseDesc {  // levels [0, n) of the single-CTA solve; level 0 is read from global memory
  int n;
  int ni[MAX_LEVELS], nj[MAX_LEVELS];
  float cx[MAX_LEVELS], cy[MAX_LEVELS];
  int off[MAX_LEVELS];  // node offset of each level in the shared arrays
  int total;
  int coarsest_sweeps;
  float omega;  // SOR factor of the coarsest level
};

__host__ __device__ inline uint8_t node_class(bool fixed, int i, int j, int ni, int nj) {
  if (fixed) return NC_FIXED;
  if (i == 0) return NC_NLEFT;
  if (i == ni - 1) return NC_NRIGHT;
  if (j == 0) return NC_NBOTTOM;
  if (j == nj - 1) return NC_NTOP;
  return NC_INTERIOR;
}

// ------------------------------------------------------------------------------------
// symmetric FP32 operator J (open-face rows scaled by 1/h): pieces shared by the
// global-memory and the shared-memory levels
// ------------------------------------------------------------------------------------
__device__ __forceinline__ float apply_J(uint8_t t, const float* y, float P, int u, int ni, float cx, float cy) {
  const float yc = y[u];
  switch (t) {
    case NC_FIXED: return yc;
    case NC_NLEFT: return cx * (y[u + 1] - yc);
    case NC_NRIGHT: return cx * (y[u - 1] - yc);
    case NC_NBOTTOM: return cy * (y[u + ni] - yc);
    case NC_NTOP: return cy * (y[u - ni] - yc);
    default: return cx * (y[u - 1] + y[u + 1] - 2.f * yc) + cy * (y[u - ni] + y[u + ni] - 2.f * yc) - P * yc;
  }
}

// Gauss-Seidel value of node u (solves its row of J y = r for y[u]).  The interior row
// divides with __fdividef (reciprocal and multiply, 2 ulp): the smoother needs no
// correctly rounded quotient, and the IEEE division's instruction sequence dominated
// the sweeps.  The diagonal 2 cx + 2 cy + P stays far below 2^126, where __fdividef
// would return 0.
__device__ __forceinline__ float gs_value(uint8_t t, const float* y, float r, float P, int u, int ni, float cx,
                                          float cy) {
  switch (t) {
    case NC_FIXED: return r;
    case NC_NLEFT: return y[u + 1] - r / cx;
    case NC_NRIGHT: return y[u - 1] - r / cx;
    case NC_NBOTTOM: return y[u + ni] - r / cy;
    case NC_NTOP: return y[u - ni] - r / cy;
    default:
      return __fdividef(cx * (y[u - 1] + y[u + 1]) + cy * (y[u - ni] + y[u + ni]) - r, 2.f * cx + 2.f * cy + P);
  }
}

// full weighting inside, injection on the boundary rows (halved: the scaled open-face
// row of a grid twice as coarse carries half the weight), zero on fixed coarse nodes
// (tf indexed at the coarse node's fine position u with row stride nif)
__device__ __forceinline__ float restrict_at(const float* tf, int u, int nif, uint8_t tc, bool edge) {
  if (tc == NC_FIXED) return 0.f;
  if (edge) return 0.5f * tf[u];
  return 0.0625f * (4.f * tf[u] + 2.f * (tf[u - 1] + tf[u + 1] + tf[u - nif] + tf[u + nif]) +
                    (tf[u - nif - 1] + tf[u - nif + 1] + tf[u + nif - 1] + tf[u + nif + 1]));
}

__device__ __forceinline__ float restrict_value(const float* tf, uint8_t tc, int I, int J, int nif, int nic, int njc) {
  return restrict_at(tf, (2 * J) * nif + 2 * I, nif, tc, I == 0 || J == 0 || I == nic - 1 || J == njc - 1);
}

// bilinear prolongation of the coarse correction yc to fine node (i, j)
__device__ __forceinline__ float prolong_value(const float* yc, int i, int j, int nic) {
  const int I = i >> 1, J = j >> 1;
  const int uc = J * nic + I;
  const bool oi = i & 1, oj = j & 1;
  if (!oi && !oj) return yc[uc];
  if (oi && !oj) return 0.5f * (yc[uc] + yc[uc + 1]);
  if (!oi && oj) return 0.5f * (yc[uc] + yc[uc + nic]);
  return 0.25f * (yc[uc] + yc[uc + 1] + yc[uc + nic] + yc[uc + nic + 1]);
}

// prolong_value from the four coarse values around fine node (i, j), already loaded:
// a = (I, J), b = (I + 1, J), c = (I, J + 1), d = (I + 1, J + 1); those outside the
// stencil are not used
__device__ __forceinline__ float prolong_of(float a, float b, float c, float d, bool oi, bool oj) {
  if (!oi && !oj) return a;
  if (oi && !oj) return 0.5f * (a + b);
  if (!oi && oj) return 0.5f * (a + c);
  return 0.25f * (a + b + c + d);
}

// ------------------------------------------------------------------------------------
// tiled V(2,2) level kernels: one launch per level on the way down (pre-smoothing from
// zero, residual, restriction) and one on the way up (prolongation, post-smoothing)
// ------------------------------------------------------------------------------------
// A block holds its TX x TY tile plus a halo of H nodes (r, P, type, y) in shared memory
// and runs the level's two red-black Gauss-Seidel sweeps there.  A half-sweep updates a
// node from its four neighbours only, so after half-sweep s the values are those of the
// global sweeps on [s, W - s) of the window: with H = 4 the tile's own nodes come out as
// in four global half-sweeps (same inputs, same arithmetic); H = 6 leaves one more ring
// for the residual and one for the full-weighting stencil.  Tiles start on even
// coordinates, so a node's colour is the parity of its window coordinates.
constexpr int TILE_NT = 256;
constexpr uint8_t TILE_OUT = 0xFF;  // window node outside the mesh

// four half-sweeps, colours first, 1 - first, first, 1 - first
template <int WX, int WY>
__device__ __forceinline__ void tile_sweeps(float* sy, const float* sr, const float* sp, const uint8_t* st, int first,
                                            float cx, float cy) {
  constexpr int NI = WX / 2 * WY;
  for (int s = 0; s < 4; s++) {
    const int color = (first + s) & 1, lo = s + 1;
#pragma unroll
    for (int k0 = 0; k0 < NI; k0 += TILE_NT) {
      const int k = k0 + threadIdx.x;
      if (k < NI) {
        const int ly = k / (WX / 2), lx = 2 * (k % (WX / 2)) + ((ly + color) & 1);
        if (lx >= lo && lx < WX - lo && ly >= lo && ly < WY - lo) {
          const int q = ly * WX + lx;
          const uint8_t t = st[q];
          if (t != TILE_OUT) sy[q] = gs_value(t, sy, sr[q], sp[q], q, WX, cx, cy);
        }
      }
    }
    __syncthreads();
  }
}

// pre-smoothing of level F from y = 0, its residual, and the restriction of that to C.r
// (every V-cycle starts each level's correction from zero, so y is not read)
template <int TX, int TY>
__device__ __forceinline__ void level_down_body(const LevelView F, const LevelView C, int bx, int by) {
  constexpr int H = 6, WX = TX + 2 * H, WY = TY + 2 * H, NW = WX * WY, NL = (NW + TILE_NT - 1) / TILE_NT;
  __shared__ float sy[NW], sr[NW], sp[NW];
  __shared__ uint8_t st[NW];
  const int gi0 = bx * TX - H, gj0 = by * TY - H;
  float vr[NL], vp[NL];
  uint8_t vt[NL];
#pragma unroll
  for (int k = 0; k < NL; k++) {
    const int q = threadIdx.x + k * TILE_NT;
    const int gi = gi0 + q % WX, gj = gj0 + q / WX;
    const bool in = q < NW && gi >= 0 && gi < F.ni && gj >= 0 && gj < F.nj;
    const int u = in ? gj * F.ni + gi : 0;
    vr[k] = F.r[u];
    vp[k] = F.P[u];
    vt[k] = in ? F.type[u] : TILE_OUT;
  }
#pragma unroll
  for (int k = 0; k < NL; k++) {
    const int q = threadIdx.x + k * TILE_NT;
    if (q < NW) {
      sy[q] = 0.f;
      sr[q] = vr[k];
      sp[q] = vp[k];
      st[q] = vt[k];
    }
  }
  __syncthreads();
  tile_sweeps<WX, WY>(sy, sr, sp, st, 0, F.cx, F.cy);
  // the tile's y into the level's scratch t: the way up reads its tile and halo from t and
  // writes y, so that no block reads a node another block of the same launch has already
  // written; and the residual on the tile plus one ring, in place of r (a node reads only
  // its own r)
  for (int k = threadIdx.x; k < TX * TY; k += TILE_NT) {
    const int gi = bx * TX + k % TX, gj = by * TY + k / TX;
    if (gi < F.ni && gj < F.nj) F.t[gj * F.ni + gi] = sy[(k / TX + H) * WX + k % TX + H];
  }
  constexpr int RX = TX + 2, RY = TY + 2;
  for (int k = threadIdx.x; k < RX * RY; k += TILE_NT) {
    const int q = (k / RX + H - 1) * WX + k % RX + H - 1;
    const uint8_t t = st[q];
    if (t != TILE_OUT) sr[q] = sr[q] - apply_J(t, sy, sp[q], q, WX, F.cx, F.cy);
  }
  __syncthreads();
  constexpr int CX = TX / 2, CY = TY / 2;
  for (int k = threadIdx.x; k < CX * CY; k += TILE_NT) {
    const int I = bx * CX + k % CX, J = by * CY + k / CX;
    if (I >= C.ni || J >= C.nj) continue;
    const int uc = J * C.ni + I;
    const int q = (2 * (k / CX) + H) * WX + 2 * (k % CX) + H;
    C.r[uc] = restrict_at(sr, q, WX, C.type[uc], I == 0 || J == 0 || I == C.ni - 1 || J == C.nj - 1);
  }
}

// F.y = F.t (the way down's y) + prolongation of C.y (not on fixed nodes), then the
// post-smoothing
template <int TX, int TY>
__device__ __forceinline__ void level_up_body(const LevelView F, const LevelView C, int bx, int by) {
  constexpr int H = 4, WX = TX + 2 * H, WY = TY + 2 * H, NW = WX * WY, NL = (NW + TILE_NT - 1) / TILE_NT;
  __shared__ float sy[NW], sr[NW], sp[NW];
  __shared__ uint8_t st[NW];
  const int gi0 = bx * TX - H, gj0 = by * TY - H;
  float vy[NL], vr[NL], vp[NL], ca[NL], cb[NL], cc[NL], cd[NL];
  uint8_t vt[NL];
#pragma unroll
  for (int k = 0; k < NL; k++) {
    const int q = threadIdx.x + k * TILE_NT;
    const int gi = gi0 + q % WX, gj = gj0 + q / WX;
    const bool in = q < NW && gi >= 0 && gi < F.ni && gj >= 0 && gj < F.nj;
    const int u = in ? gj * F.ni + gi : 0;
    vy[k] = F.t[u];
    vr[k] = F.r[u];
    vp[k] = F.P[u];
    vt[k] = in ? F.type[u] : TILE_OUT;
    const int I = in ? gi >> 1 : 0, J = in ? gj >> 1 : 0;
    const int I1 = min(I + 1, C.ni - 1), J1 = min(J + 1, C.nj - 1);
    ca[k] = C.y[J * C.ni + I];
    cb[k] = C.y[J * C.ni + I1];
    cc[k] = C.y[J1 * C.ni + I];
    cd[k] = C.y[J1 * C.ni + I1];
  }
#pragma unroll
  for (int k = 0; k < NL; k++) {
    const int q = threadIdx.x + k * TILE_NT;
    if (q < NW) {
      const int gi = gi0 + q % WX, gj = gj0 + q / WX;
      float y = vy[k];
      if (vt[k] != TILE_OUT && vt[k] != NC_FIXED) y += prolong_of(ca[k], cb[k], cc[k], cd[k], gi & 1, gj & 1);
      sy[q] = y;
      sr[q] = vr[k];
      sp[q] = vp[k];
      st[q] = vt[k];
    }
  }
  __syncthreads();
  tile_sweeps<WX, WY>(sy, sr, sp, st, 1, F.cx, F.cy);
  for (int k = threadIdx.x; k < TX * TY; k += TILE_NT) {
    const int gi = bx * TX + k % TX, gj = by * TY + k / TX;
    if (gi < F.ni && gj < F.nj) F.y[gj * F.ni + gi] = sy[(k / TX + H) * WX + k % TX + H];
  }
}

template <int TX, int TY>
__global__ void __launch_bounds__(TILE_NT) k_level_down(LevelView F, LevelView C) {
  level_down_body<TX, TY>(F, C, blockIdx.x, blockIdx.y);
}

template <int TX, int TY>
__global__ void __launch_bounds__(TILE_NT) k_level_up(LevelView F, LevelView C) {
  level_up_body<TX, TY>(F, C, blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------------------------------
// coarse-grid P: injection of the fine linearisation coefficient
__global__ void k_restrict_P(LevelView F, LevelView Cl) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= Cl.ni || J >= Cl.nj) return;
  Cl.P[J * Cl.ni + I] = F.P[(2 * J) * F.ni + 2 * I];
}

// ------------------------------------------------------------------------------------
// single-CTA V-cycle over the coarse end of the hierarchy (shared memory)
// ------------------------------------------------------------------------------------
// rb: red then black (pre-smoothing); otherwise black then red (post-smoothing), so the
// V-cycle is a symmetric preconditioner
__device__ void cta_smooth(float* y, const float* r, const float* P, const uint8_t* ty, int ni, int nj, float cx,
                           float cy, int sweeps, bool rb, float omega = 1.f) {
  const int n = ni * nj;
  const bool sor = omega != 1.f;  // Gauss-Seidel stores the value itself, as the level kernels do
  for (int s = 0; s < sweeps; s++)
    for (int c = 0; c < 2; c++) {
      const int color = rb ? c : 1 - c;
      if (ni & 1) {
        // odd row length: the colour (i + j) & 1 of node u = j ni + i is u & 1
        for (int u = 2 * threadIdx.x + color; u < n; u += 2 * blockDim.x) {
          const float g = gs_value(ty[u], y, r[u], P[u], u, ni, cx, cy);
          y[u] = sor ? y[u] + omega * (g - y[u]) : g;
        }
      } else {
        for (int u = threadIdx.x; u < n; u += blockDim.x) {
          const int j = u / ni, i = u - j * ni;
          if (((i + j) & 1) != color) continue;
          const float g = gs_value(ty[u], y, r[u], P[u], u, ni, cx, cy);
          y[u] = sor ? y[u] + omega * (g - y[u]) : g;
        }
      }
      __syncthreads();
    }
}

__device__ __forceinline__ void coarse_vcycle_body(const CoarseDesc& D, const LevelView& top, int nu1, int nu2) {
  extern __shared__ __align__(16) unsigned char sm[];
  float* Y = reinterpret_cast<float*>(sm);
  float* R = Y + D.total;
  float* PP = R + D.total;
  float* T = PP + D.total;
  uint8_t* TY = reinterpret_cast<uint8_t*>(T + D.total);
  const int n0 = D.ni[0] * D.nj[0];
  // top level in: eight loads per thread in flight at a time
  for (int u0 = 0; u0 < n0; u0 += 8 * blockDim.x) {
    float rr[8], pp[8];
    uint8_t tt[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int u = u0 + threadIdx.x + k * blockDim.x, uu = u < n0 ? u : 0;
      rr[k] = top.r[uu];
      pp[k] = top.P[uu];
      tt[k] = top.type[uu];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int u = u0 + threadIdx.x + k * blockDim.x;
      if (u < n0) {
        Y[u] = 0.f;
        R[u] = rr[k];
        PP[u] = pp[k];
        TY[u] = tt[k];
      }
    }
  }
  __syncthreads();
  // coarser levels: type and P by injection
  for (int l = 1; l < D.n; l++) {
    const int nic = D.ni[l], njc = D.nj[l], nif = D.ni[l - 1];
    const int oc = D.off[l], of = D.off[l - 1];
    for (int u = threadIdx.x; u < nic * njc; u += blockDim.x) {
      const int J = u / nic, I = u - J * nic;
      const int uf = of + (2 * J) * nif + 2 * I;
      TY[oc + u] = node_class(TY[uf] == NC_FIXED, I, J, nic, njc);
      PP[oc + u] = PP[uf];
    }
    __syncthreads();
  }
  // descend
  for (int l = 0; l < D.n - 1; l++) {
    const int o = D.off[l], ni = D.ni[l], nj = D.nj[l];
    cta_smooth(Y + o, R + o, PP + o, TY + o, ni, nj, D.cx[l], D.cy[l], nu1, true);
    for (int u = threadIdx.x; u < ni * nj; u += blockDim.x)
      T[o + u] = R[o + u] - apply_J(TY[o + u], Y + o, PP[o + u], u, ni, D.cx[l], D.cy[l]);
    __syncthreads();
    const int oc = D.off[l + 1], nic = D.ni[l + 1], njc = D.nj[l + 1];
    for (int u = threadIdx.x; u < nic * njc; u += blockDim.x) {
      const int J = u / nic, I = u - J * nic;
      R[oc + u] = restrict_value(T + o, TY[oc + u], I, J, ni, nic, njc);
      Y[oc + u] = 0.f;
    }
    __syncthreads();
  }
  // coarsest: symmetric pairs of red-black SOR sweeps with the optimal Laplacian omega
  // (a coarsest grid of tens of nodes per side, left when n - 1 has an odd factor,
  // needs it: plain Gauss-Seidel would barely reduce its error)
  {
    const int l = D.n - 1, o = D.off[l];
    for (int s = 0; s < D.coarsest_sweeps; s++) {
      cta_smooth(Y + o, R + o, PP + o, TY + o, D.ni[l], D.nj[l], D.cx[l], D.cy[l], 1, true, D.omega);
      cta_smooth(Y + o, R + o, PP + o, TY + o, D.ni[l], D.nj[l], D.cx[l], D.cy[l], 1, false, D.omega);
    }
  }
  // ascend
  for (int l = D.n - 2; l >= 0; l--) {
    const int o = D.off[l], ni = D.ni[l], nj = D.nj[l];
    const int oc = D.off[l + 1], nic = D.ni[l + 1];
    for (int u = threadIdx.x; u < ni * nj; u += blockDim.x) {
      if (TY[o + u] == NC_FIXED) continue;
      const int j = u / ni, i = u - j * ni;
      Y[o + u] += prolong_value(Y + oc, i, j, nic);
    }
    __syncthreads();
    cta_smooth(Y + o, R + o, PP + o, TY + o, ni, nj, D.cx[l], D.cy[l], nu2, false);
  }
  for (int u = threadIdx.x; u < n0; u += blockDim.x) top.y[u] = Y[u];
}

__global__ void __launch_bounds__(1024, 1) k_coarse_vcycle(CoarseDesc D, LevelView top, int nu1, int nu2) {
  coarse_vcycle_body(D, top, nu1, nu2);
}

// ------------------------------------------------------------------------------------
// FP64 outer loop
// ------------------------------------------------------------------------------------
struct NlArgs {
  int ni, nj;
  double cx, cy, dx, dy;  // 1/dx^2, 1/dy^2, dx, dy
  double C_n0;            // (e/eps) n0
  double inv_kTe, phi0;
  int linear;
  int fp64_exp;  // 0: Boltzmann exponential in FP32 (with an error bound), 1: FP64
  // axisymmetric meshes: 1 = RZ (radius along i), 2 = ZR (radius along j), 0 = XY;
  // r0, dr: radius of the first node column / row and its spacing
  int axi = 0;
  double r0 = 0.0, dr = 0.0;
};

constexpr int RB = 256;

__device__ inline void block_sum2(double a, double b, double* part, bool max2, int bidx) {
  __shared__ double sh[2][RB / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    const double bb = __shfl_down_sync(0xffffffffu, b, o);
    b = max2 ? fmax(b, bb) : b + bb;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][wid] = a;
    sh[1][wid] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0, y = 0;
    for (int w = 0; w < RB / 32; w++) {
      x += sh[0][w];
      y = max2 ? fmax(y, sh[1][w]) : y + sh[1][w];
    }
    part[2 * bidx] = x;
    part[2 * bidx + 1] = y;
  }
}

// per block: sum of a, max of b, max of c -> part[3 * block + {0, 1, 2}]
__device__ inline void block_sum_max_max(double a, double b, double c, double* part, int bidx) {
  __shared__ double sh[3][RB / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b = fmax(b, __shfl_down_sync(0xffffffffu, b, o));
    c = fmax(c, __shfl_down_sync(0xffffffffu, c, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][wid] = a;
    sh[1][wid] = b;
    sh[2][wid] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0, y = 0, z = 0;
    for (int w = 0; w < RB / 32; w++) {
      x += sh[0][w];
      y = fmax(y, sh[1][w]);
      z = fmax(z, sh[2][w]);
    }
    part[3 * bidx] = x;
    part[3 * bidx + 1] = y;
    part[3 * bidx + 2] = z;
  }
}

// exp(x) for |x| <= 700 by Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point arithmetic", ACM TOMS
// 15(2), 1989): x = (64 m + j) ln2/64 + r with |r| <= ln2/128, and
// exp(x) = 2^m 2^(j/64) (1 + r + r q(r)),  q(r) = r/2 + r^2/6 + r^3/24.
// q is evaluated in FP32: its relative rounding (a few 2^-24) on a value of at most
// ln2/256 changes the result by under 3e-12 relative; the truncated series by 4e-14; the
// reduction (one FMA with ln2/64 rounded to FP64) by under 1e-13 for |x| <= 700.  So the
// result is within 5e-12 relative of exp(x), with four FP64 operations where the FP64
// exponential takes many more -- the Newton residual is bound by the FP64 pipe.  Outside
// [-700, 700] (and for NaN) it is the FP64 exponential.
__device__ const double d_exp2_j64[64] = {
    1.0, 1.0108892860517005, 1.0218971486541166, 1.0330248790212284,
    1.0442737824274138, 1.0556451783605572, 1.0671404006768237, 1.0787607977571199,
    1.0905077326652577, 1.102382583307841, 1.1143867425958924, 1.1265216186082418,
    1.1387886347566916, 1.1511892299529827, 1.1637248587775775, 1.1763969916502812,
    1.189207115002721, 1.202156731452703, 1.215247359980469, 1.22848053610687,
    1.241857812073484, 1.255380757024691, 1.2690509571917332, 1.2828700160787783,
    1.2968395546510096, 1.3109612115247644, 1.3252366431597413, 1.339667524053303,
    1.3542555469368927, 1.3690024229745905, 1.383909881963832, 1.3989796725383112,
    1.4142135623730951, 1.42961333839197, 1.4451808069770467, 1.460917794180647,
    1.4768261459394993, 1.4929077282912648, 1.5091644275934228, 1.5255981507445384,
    1.5422108254079407, 1.559004400237837, 1.5759808451078865, 1.593142151342267,
    1.6104903319492543, 1.6280274218573478, 1.645755478153965, 1.6636765803267364,
    1.681792830507429, 1.7001063537185235, 1.718619298122478, 1.7373338352737062,
    1.7562521603732995, 1.7753764925265212, 1.7947090750031072, 1.8142521755003989,
    1.8340080864093424, 1.8539791250833855, 1.8741676341103, 1.8945759815869656,
    1.9152065613971474, 1.9360617934922943, 1.9571441241754002, 1.978456026387951};
__device__ __forceinline__ double exp_tang(double x) {
  if (!(fabs(x) <= 700.0)) return exp(x);
  const int n = __double2int_rn(x * 92.33248261689366);  // 64 / ln 2
  const double r = fma((double)(-n), 0.010830424696249145, x);  // ln 2 / 64
  const float rf = (float)r;
  const float q = rf * fmaf(rf, fmaf(rf, 1.f / 24.f, 1.f / 6.f), 0.5f);
  const double p = fma(r, (double)q, r);
  const double t = __ldg(&d_exp2_j64[n & 63]);
  const double e = fma(t, p, t);  // in [0.99, 2): a normal number
  return __longlong_as_double(__double_as_longlong(e) + ((long long)(n >> 6) << 52));
}

// F = A x - b0 - (e n0/eps) exp((x - phi0)/kTe) on interior rows, x - bc on fixed rows,
// the one-sided gradient on open-face rows (b = 0 there, as Solver.java:322-338 sets);
// P = d(exp term)/dx.  F (open-face rows scaled by 1/h for the symmetric inner system)
// and P go to the FP32 level 0; per block sum F^2, max |F| of the unscaled F and the
// largest error bound of an FP32 exponential.
// The Laplacian is FP64 (its terms cancel to ~1e-14 of their size at the tolerance);
// the Boltzmann term is small next to them and is taken in FP32 (exponential, its
// coefficient and P; the FP64 pipe is the kernel's bound) unless a.fp64_exp or its
// value leaves the FP32 range: its relative error is at most |arg| 2^-24 (rounding of
// the argument) plus 2^-22 (expf) plus 2^-23 (the FP32 coefficient and product), and the
// host switches to FP64 when that bound could reach the tolerance.  The FP64 form is
// exp_tang: its 5e-12 relative error adds at most 5e-12 times the largest Boltzmann term
// over sqrt(N) to ||R||_2 / N (1e-11 for e n0/eps = 1.8e4 on a 2049x1025 mesh).
// Blocks bidx = 0..G-1 of one mesh (the single and the batched launch share it, so that
// the partial sums, and with them every reduction, are the same bit for bit).
__device__ __forceinline__ void nl_residual_body(const NlArgs& a, const double* __restrict__ x,
                                                 const double* __restrict__ b0, const uint8_t* __restrict__ type,
                                                 float* __restrict__ F32, float* __restrict__ P32,
                                                 double* __restrict__ partial, int bidx, int G) {
  const int n = a.ni * a.nj;
  const float Cf = (float)a.C_n0, kf = (float)a.inv_kTe;
  double s2 = 0.0, smax = 0.0;
  float emax = 0.f;
  for (int u = bidx * RB + threadIdx.x; u < n; u += G * RB) {
    const uint8_t t = type[u];
    const double xc = x[u];
    double F, Fs;
    float P = 0.f;
    // axisymmetric: the radius of the node's row (ZR) or column (RZ) and of the faces
    // half a cell below / above it; the inner system's row weights (symmetric form)
    double rc = 1.0, rm = 1.0, rp = 1.0;
    if (a.axi) {
      const int k = a.axi == 1 ? u % a.ni : u / a.ni;
      rc = a.r0 + k * a.dr;
      rm = rc - 0.5 * a.dr;
      rp = rc + 0.5 * a.dr;
    }
    switch (t) {
      case NC_FIXED: F = Fs = xc - b0[u]; break;
      case NC_NLEFT: F = (x[u + 1] - xc) / a.dx; Fs = F / a.dx * (a.axi == 1 ? rp : rc); break;
      case NC_NRIGHT: F = (xc - x[u - 1]) / a.dx; Fs = -F / a.dx * (a.axi == 1 ? rm : rc); break;
      case NC_NBOTTOM: F = (x[u + a.ni] - xc) / a.dy; Fs = F / a.dy * (a.axi == 2 ? rp : rc); break;
      case NC_NTOP: F = (xc - x[u - a.ni]) / a.dy; Fs = -F / a.dy * (a.axi == 2 ? rm : rc); break;
      default: {
        // XY: the 5-point operator.  RZ / ZR: the reference's FVM row on the uniform mesh
        // (Solver.java:451-553: face fluxes weighted by the face radius, divided by the
        // node volume 2 pi r dA), i.e. the cylindrical Laplacian / 2 pi
        double Ax;
        if (a.axi == 2)
          Ax = (rc * a.cx * (x[u - 1] + x[u + 1] - 2.0 * xc) +
                a.cy * (rp * (x[u + a.ni] - xc) + rm * (x[u - a.ni] - xc))) / (2.0 * PI * rc);
        else if (a.axi == 1)
          Ax = (a.cx * (rp * (x[u + 1] - xc) + rm * (x[u - 1] - xc)) +
                rc * a.cy * (x[u - a.ni] + x[u + a.ni] - 2.0 * xc)) / (2.0 * PI * rc);
        else
          Ax = a.cx * (x[u - 1] + x[u + 1] - 2.0 * xc) + a.cy * (x[u - a.ni] + x[u + a.ni] - 2.0 * xc);
        double ex = 0.0;
        if (!a.linear) {
          const double arg = (xc - a.phi0) * a.inv_kTe;
          const float argf = (float)arg;
          const float exf = (a.fp64_exp || arg > 80.0) ? INFINITY : Cf * expf(argf);
          if (exf <= 3.0e38f) {
            ex = (double)exf;
            P = exf * kf;
            emax = fmaxf(emax, exf * (fabsf(argf) * 5.9604645e-8f + 3.5762787e-7f));
          } else {
            ex = a.C_n0 * exp_tang(arg);
            P = (float)(ex * a.inv_kTe);
          }
        }
        F = Fs = Ax - (b0[u] + ex);
        if (a.axi) {
          // the symmetric inner system: this row times 2 pi r, and P likewise (per unit r)
          Fs = 2.0 * PI * rc * F;
          P *= (float)(2.0 * PI);
        }
      }
    }
    F32[u] = (float)Fs;
    P32[u] = P;
    s2 += F * F;
    smax = fmax(smax, fabs(F));
  }
  block_sum_max_max(s2, smax, (double)emax, partial, bidx);
}

__global__ void __launch_bounds__(RB) k_nl_residual(NlArgs a, const double* __restrict__ x,
                                                    const double* __restrict__ b0, const uint8_t* __restrict__ type,
                                                    float* __restrict__ F32, float* __restrict__ P32,
                                                    double* __restrict__ partial) {
  nl_residual_body(a, x, b0, type, F32, P32, partial, blockIdx.x, gridDim.x);
}

// one block of 256 threads
__device__ __forceinline__ void reduce3_body(const double* partial, int nb, double* out) {
  __shared__ double sa[256], sb[256], sc[256];
  double a = 0, b = 0, c = 0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    a += partial[3 * k];
    b = fmax(b, partial[3 * k + 1]);
    c = fmax(c, partial[3 * k + 2]);
  }
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sa[threadIdx.x] += sa[threadIdx.x + w];
      sb[threadIdx.x] = fmax(sb[threadIdx.x], sb[threadIdx.x + w]);
      sc[threadIdx.x] = fmax(sc[threadIdx.x], sc[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sa[0];
    out[1] = sb[0];
    out[2] = sc[0];
  }
}

__global__ void k_reduce_partials3(const double* partial, int nb, double* out) { reduce3_body(partial, nb, out); }

// one block of 256 threads
__device__ __forceinline__ void reduce2_body(const double* partial, int nb, double* out, int max2) {
  __shared__ double s2[256], sm[256];
  double a2 = 0, am = 0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    a2 += partial[2 * b];
    am = max2 ? fmax(am, partial[2 * b + 1]) : am + partial[2 * b + 1];
  }
  s2[threadIdx.x] = a2;
  sm[threadIdx.x] = am;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s2[threadIdx.x] += s2[threadIdx.x + w];
      sm[threadIdx.x] = max2 ? fmax(sm[threadIdx.x], sm[threadIdx.x + w]) : sm[threadIdx.x] + sm[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s2[0];
    out[1] = sm[0];
  }
}

__global__ void k_reduce_partials(const double* partial, int nb, double* out, int max2) {
  reduce2_body(partial, nb, out, max2);
}

// ---- flexible preconditioned CG on J y = F (FP32 vectors, FP64 dot products) -------
// scalars: sc[0] = r.z, sc[1] = p.Jp, sc[2] = alpha, sc[3] = beta, sc[4..5] = reduction out
enum { SC_RZ = 0, SC_PQ = 1, SC_ALPHA = 2, SC_BETA = 3, SC_RED = 4 };

// q = J p and the partial sums of p.q
__device__ __forceinline__ void cg_matvec_body(const LevelView& L, const float* __restrict__ p, float* __restrict__ q,
                                               double* __restrict__ partial, int bidx, int G) {
  const int n = L.ni * L.nj;
  float s = 0.f;  // a thread sums a few dozen products; blocks and the grid sum in FP64
  for (int u = bidx * RB + threadIdx.x; u < n; u += G * RB) {
    const float qu = apply_J(L.type[u], p, L.P[u], u, L.ni, L.cx, L.cy);
    q[u] = qu;
    s = fmaf(p[u], qu, s);
  }
  block_sum2((double)s, 0.0, partial, false, bidx);
}

__global__ void __launch_bounds__(RB) k_cg_matvec(LevelView L, const float* __restrict__ p, float* __restrict__ q,
                                                  double* __restrict__ partial) {
  cg_matvec_body(L, p, q, partial, blockIdx.x, gridDim.x);
}

// row-weighted J of an axisymmetric mesh (see AxiView); P is stored as 2 pi P
__device__ __forceinline__ float apply_Jw(uint8_t t, const float* y, float P, int u, int ni, float cx, float cy,
                                          const AxiView& X) {
  const float yc = y[u];
  const int k = X.axi == 1 ? u % ni : u / ni;
  const float rc = X.r0 + (float)k * X.dr, rm = rc - 0.5f * X.dr, rp = rc + 0.5f * X.dr;
  switch (t) {
    case NC_FIXED: return yc;
    case NC_NLEFT: return (X.axi == 1 ? rp : rc) * cx * (y[u + 1] - yc);
    case NC_NRIGHT: return (X.axi == 1 ? rm : rc) * cx * (y[u - 1] - yc);
    case NC_NBOTTOM: return (X.axi == 2 ? rp : rc) * cy * (y[u + ni] - yc);
    case NC_NTOP: return (X.axi == 2 ? rm : rc) * cy * (y[u - ni] - yc);
    default:
      if (X.axi == 2)
        return rc * cx * (y[u - 1] + y[u + 1] - 2.f * yc) + cy * (rp * (y[u + ni] - yc) + rm * (y[u - ni] - yc)) -
               rc * P * yc;
      return cx * (rp * (y[u + 1] - yc) + rm * (y[u - 1] - yc)) + rc * cy * (y[u - ni] + y[u + ni] - 2.f * yc) -
             rc * P * yc;
  }
}

__global__ void __launch_bounds__(RB) k_cg_matvec_axi(LevelView L, AxiView X, const float* __restrict__ p,
                                                      float* __restrict__ q, double* __restrict__ partial) {
  const int n = L.ni * L.nj;
  float s = 0.f;
  for (int u = blockIdx.x * RB + threadIdx.x; u < n; u += gridDim.x * RB) {
    const float qu = apply_Jw(L.type[u], p, L.P[u], u, L.ni, L.cx, L.cy, X);
    q[u] = qu;
    s = fmaf(p[u], qu, s);
  }
  block_sum2((double)s, 0.0, partial, false, blockIdx.x);
}

// The preconditioner of the row-weighted system: z = D^-1/2 V(D^-1/2 r) with D the row
// radii (a quarter cell on the axis) and V the XY multigrid cycle on the level-0 P (which
// holds 2 pi P): D^-1/2 J_w D^-1/2 is the XY operator up to terms of order (dr / r)^2.
__device__ __forceinline__ float axi_scale(const AxiView& X, int u, int ni) {
  const int k = X.axi == 1 ? u % ni : u / ni;
  return rsqrtf(fmaxf(X.r0 + (float)k * X.dr, 0.25f * X.dr));
}
__global__ void k_axi_pre(LevelView L, AxiView X, float* __restrict__ keep) {
  const int n = L.ni * L.nj;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const float ru = L.r[u];
    keep[u] = ru;
    L.r[u] = axi_scale(X, u, L.ni) * ru;
  }
}
__global__ void k_axi_post(LevelView L, AxiView X, const float* __restrict__ keep) {
  const int n = L.ni * L.nj;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    L.y[u] *= axi_scale(X, u, L.ni);
    L.r[u] = keep[u];
  }
}

// Coarse correction by the network inside the first preconditioner application of a
// Newton step: keep r, then r <- r - J e (e: the network's correction).
__global__ void k_pc_residual(LevelView L, const float* __restrict__ e, float* __restrict__ keep) {
  const int n = L.ni * L.nj;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const float ru = L.r[u];
    keep[u] = ru;
    L.r[u] = ru - apply_J(L.type[u], e, L.P[u], u, L.ni, L.cx, L.cy);
  }
}
// ... after the V-cycle on r - J e: z <- V(r - J e) + e, r restored
__global__ void k_pc_finish(LevelView L, const float* __restrict__ e, const float* __restrict__ keep) {
  const int n = L.ni * L.nj;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    L.y[u] += e[u];
    L.r[u] = keep[u];
  }
}

// x += alpha p, r -= alpha q, zo = z
__device__ __forceinline__ void cg_axpy_node(int u, float al, const float* __restrict__ p, const float* __restrict__ q,
                                             float* __restrict__ x, float* __restrict__ r, const float* __restrict__ z,
                                             float* __restrict__ zo) {
  x[u] += al * p[u];
  r[u] -= al * q[u];
  zo[u] = z[u];
}

__global__ void k_cg_axpy(int n, const double* __restrict__ sc, const float* __restrict__ p, const float* __restrict__ q,
                          float* __restrict__ x, float* __restrict__ r, const float* __restrict__ z, float* __restrict__ zo) {
  const float al = (float)sc[SC_ALPHA];
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
    cg_axpy_node(u, al, p, q, x, r, z, zo);
}

// partial sums of r.z and r.(z - zo)
__device__ __forceinline__ void cg_dots_body(int n, const float* __restrict__ r, const float* __restrict__ z,
                                             const float* __restrict__ zo, double* __restrict__ partial, int bidx,
                                             int G) {
  float a = 0.f, b = 0.f;  // per-thread FP32, blocks and the grid in FP64
  for (int u = bidx * RB + threadIdx.x; u < n; u += G * RB) {
    const float ru = r[u], zu = z[u];
    a = fmaf(ru, zu, a);
    b = fmaf(ru, zu - zo[u], b);
  }
  block_sum2((double)a, (double)b, partial, false, bidx);
}

__global__ void __launch_bounds__(RB) k_cg_dots(int n, const float* __restrict__ r, const float* __restrict__ z,
                                                const float* __restrict__ zo, double* __restrict__ partial) {
  cg_dots_body(n, r, z, zo, partial, blockIdx.x, gridDim.x);
}

// scalar updates of the CG recurrence (one thread)
__device__ __forceinline__ void cg_scalars_body(double* sc, int stage) {
  if (stage == 0) {            // after the first preconditioning: rz = r.z
    sc[SC_RZ] = sc[SC_RED];
  } else if (stage == 1) {     // after p.q: alpha = rz / pq
    sc[SC_PQ] = sc[SC_RED];
    sc[SC_ALPHA] = (sc[SC_PQ] != 0.0) ? sc[SC_RZ] / sc[SC_PQ] : 0.0;
  } else {                     // after r.z, r.(z-zo): Polak-Ribiere beta, new rz
    sc[SC_BETA] = (sc[SC_RZ] != 0.0) ? sc[SC_RED + 1] / sc[SC_RZ] : 0.0;
    sc[SC_RZ] = sc[SC_RED];
  }
}

__global__ void k_cg_scalars(double* sc, int stage) {
  if (threadIdx.x == 0) cg_scalars_body(sc, stage);
}

// p = z + beta p; the first direction is z itself (p holds no value yet: not even its
// product with 0 may be formed, it could be a NaN pattern)
__device__ __forceinline__ void cg_pupdate_node(int u, int first, float be, const float* __restrict__ z,
                                                float* __restrict__ p) {
  p[u] = first ? z[u] : z[u] + be * p[u];
}

__global__ void k_cg_pupdate(int n, const double* __restrict__ sc, int first, const float* __restrict__ z,
                             float* __restrict__ p) {
  const float be = first ? 0.f : (float)sc[SC_BETA];
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
    cg_pupdate_node(u, first, be, z, p);
}

// x -= y, each node's step limited to max_step (10 kTe): far from the solution an
// undamped Newton step on the exponential can overshoot into overflow; near it the
// steps are tiny and the limit never acts, so the converged potential is unchanged
__device__ __forceinline__ void update_phi_node(int u, double* __restrict__ x, const float* __restrict__ y,
                                                double max_step) {
  x[u] -= fmin(fmax((double)y[u], -max_step), max_step);
}

__global__ void k_update_phi(int n, double* __restrict__ x, const float* __restrict__ y, double max_step) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
    update_phi_node(u, x, y, max_step);
}

__device__ __forceinline__ double b0_value(uint8_t t, double bc, double rho, double inv_eps) {
  return (t == NC_FIXED) ? bc : (t == NC_INTERIOR ? -rho * inv_eps : 0.0);
}

__global__ void k_build_b0(int n, const double* __restrict__ rho, const double* __restrict__ bc,
                           const uint8_t* __restrict__ type, double inv_eps, double* __restrict__ b0) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
    b0[u] = b0_value(type[u], bc[u], rho[u], inv_eps);
}

__global__ void k_fix_phi(int n, double* __restrict__ x, const double* __restrict__ bc, const uint8_t* __restrict__ type) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
    if (type[u] == NC_FIXED) x[u] = bc[u];
}

// E = -grad(phi): central differences inside, one-sided on the mesh edges
// (the rows Solver.getNodeGradient assembles, Solver.java:559-611)
__device__ __forceinline__ void efield_node(int u, int ni, int nj, double inv_dx, double inv_dy,
                                            const double* __restrict__ phi, double* __restrict__ efi,
                                            double* __restrict__ efj, float4* __restrict__ E) {
  {
    const int j = u / ni, i = u - j * ni;
    double gi, gj;
    if (i == 0) gi = (phi[u + 1] - phi[u]) * inv_dx;
    else if (i == ni - 1) gi = (phi[u] - phi[u - 1]) * inv_dx;
    else gi = (phi[u + 1] - phi[u - 1]) * (0.5 * inv_dx);
    if (j == 0) gj = (phi[u + ni] - phi[u]) * inv_dy;
    else if (j == nj - 1) gj = (phi[u] - phi[u - ni]) * inv_dy;
    else gj = (phi[u + ni] - phi[u - ni]) * (0.5 * inv_dy);
    efi[u] = -gi;
    efj[u] = -gj;
    store_efield(E, u, make_float2((float)(-gi), (float)(-gj)));
  }
}

__global__ void k_efield(int ni, int nj, double inv_dx, double inv_dy, const double* __restrict__ phi,
                         double* __restrict__ efi, double* __restrict__ efj, float4* __restrict__ E) {
  const int n = ni * nj;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
    efield_node(u, ni, nj, inv_dx, inv_dy, phi, efi, efj, E);
}

__global__ void k_boltzmann(int n, const double* __restrict__ phi, double n0, double inv_kTe, double phi0,
                            double* __restrict__ ne) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    double d = n0 * exp((phi[u] - phi0) * inv_kTe);
    ne[u] = d < 1.0 ? 1.0 : d;
  }
}

__device__ __forceinline__ double rho_add(double acc, double q, double nd) { return acc + q * nd; }

__global__ void k_rho_add(int n, const double* __restrict__ nd, double q, double* __restrict__ rho) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) rho[u] = rho_add(rho[u], q, nd[u]);
}

}  // namespace

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
struct SfPoisson {
  int ni = 0, nj = 0;
  double *phi = nullptr, *b0 = nullptr, *rho = nullptr, *bc = nullptr, *ne = nullptr;
  double *efi = nullptr, *efj = nullptr, *partial = nullptr, *red = nullptr, *sc = nullptr;
  float *cg_x = nullptr, *cg_p = nullptr, *cg_q = nullptr, *cg_zo = nullptr;
  uint8_t* type0 = nullptr;
  std::vector<LevelView> lv;
  std::vector<void*> allocs;
  int cs = 0;  // first level of the single-CTA solve
  CoarseDesc cd{};
  size_t coarse_smem = 0;
  int cs_b = 0;  // the same for the batched solve
  CoarseDesc cd_b{};
  size_t coarse_smem_b = 0;
  int red_blocks = 0;
  bool rho_set = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  sf_poisson_params prm{};
  bool have_prm = false;
  bool fp64_exp = false;  // a previous solve needed the FP64 exponential: start there
  // the inner work of one Newton step (restrict P, PCG, update) as a CUDA graph; [1] the
  // step that applies the network's coarse correction, [0] the plain one
  cudaGraphExec_t step_graph[2] = {nullptr, nullptr};
  int graph_iters[2] = {-1, -1};
  double graph_max_step[2] = {0, 0};
  int64_t graph_launches[2] = {0, 0};
  // axisymmetric meshes (0 for XY)
  int axi = 0;
  AxiView axv{};
  double r0 = 0.0, dr = 0.0;
  float* axi_keep = nullptr;
};

// zeroed: the first solve without a host phi starts from phi = 0, and no buffer holds
// stale bit patterns from earlier allocations
static void* dalloc(sf_ctx* ctx, SfPoisson* ps, size_t bytes) {
  void* p = nullptr;
  SF_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
  ps->allocs.push_back(p);
  zero_wait(p, std::max<size_t>(bytes, 16), ctx->stream);
  return p;
}

static SfPoisson* poisson_get(sf_ctx* ctx) {
  if (ctx->poisson) return ctx->poisson;
  const int axi = ctx->domain == SF_DOMAIN_RZ ? 1 : (ctx->domain == SF_DOMAIN_ZR ? 2 : 0);
  SF_REQUIRE(!axi || ctx->x0[axi - 1] >= 0.0, SF_ERR_ARG, "axisymmetric mesh with negative radii");
  SfPoisson* ps = new SfPoisson();
  ctx->poisson = ps;
  ps->axi = axi;
  if (axi) {
    ps->r0 = ctx->x0[axi - 1];
    ps->dr = ctx->dh[axi - 1];
    ps->axv = AxiView{axi, (float)ps->r0, (float)ps->dr};
  }
  const int ni = ctx->ni, nj = ctx->nj;
  const size_t nn = (size_t)ni * nj;
  ps->ni = ni;
  ps->nj = nj;
  ps->phi = (double*)dalloc(ctx, ps, 8 * nn);
  ps->b0 = (double*)dalloc(ctx, ps, 8 * nn);
  ps->rho = (double*)dalloc(ctx, ps, 8 * nn);
  ps->bc = (double*)dalloc(ctx, ps, 8 * nn);
  ps->ne = (double*)dalloc(ctx, ps, 8 * nn);
  ps->efi = (double*)dalloc(ctx, ps, 8 * nn);
  ps->efj = (double*)dalloc(ctx, ps, 8 * nn);
  ps->cg_x = (float*)dalloc(ctx, ps, 4 * nn);
  ps->cg_p = (float*)dalloc(ctx, ps, 4 * nn);
  ps->cg_q = (float*)dalloc(ctx, ps, 4 * nn);
  ps->cg_zo = (float*)dalloc(ctx, ps, 4 * nn);
  if (axi) ps->axi_keep = (float*)dalloc(ctx, ps, 4 * nn);
  ps->type0 = (uint8_t*)dalloc(ctx, ps, nn);
  // the partition of every reduction depends on the mesh alone (a batched solve of the
  // same mesh reproduces the sums bit for bit)
  ps->red_blocks = std::min<int>(ctx->num_sms * 4, (int)((nn + RB - 1) / RB));
  ps->partial = (double*)dalloc(ctx, ps, 24 * (size_t)ps->red_blocks);
  ps->red = (double*)dalloc(ctx, ps, 24);
  ps->sc = (double*)dalloc(ctx, ps, 8 * 8);
  SF_CUDA(cudaMemsetAsync(ps->phi, 0, 8 * nn, ctx->stream));
  SF_CUDA(cudaMemsetAsync(ps->rho, 0, 8 * nn, ctx->stream));
  SF_CUDA(cudaMemcpyAsync(ps->bc, ctx->bc_value.data(), 8 * nn, cudaMemcpyHostToDevice, ctx->stream));
  // node classes of the fine level (fixed = Dirichlet or internal nodes, Mesh.isDirichletNode)
  std::vector<uint8_t> t0(nn);
  for (int j = 0; j < nj; j++)
    for (int i = 0; i < ni; i++) {
      const int nt = ctx->node_type[(size_t)j * ni + i];
      t0[(size_t)j * ni + i] = node_class(nt == SF_NODE_DIRICHLET || nt == SF_NODE_INTERNAL, i, j, ni, nj);
    }
  SF_CUDA(cudaMemcpyAsync(ps->type0, t0.data(), nn, cudaMemcpyHostToDevice, ctx->stream));
  // multigrid hierarchy: halve while both node counts are odd (2m+1) and >= 5
  std::vector<std::vector<uint8_t>> types;
  types.push_back(t0);
  int lni = ni, lnj = nj;
  double ldx = ctx->dh[0], ldy = ctx->dh[1];
  for (int l = 0; l < MAX_LEVELS; l++) {
    LevelView L;
    L.ni = lni;
    L.nj = lnj;
    L.cx = (float)(1.0 / (ldx * ldx));
    L.cy = (float)(1.0 / (ldy * ldy));
    const size_t n = (size_t)lni * lnj;
    L.y = (float*)dalloc(ctx, ps, 4 * n);
    L.r = (float*)dalloc(ctx, ps, 4 * n);
    L.P = (float*)dalloc(ctx, ps, 4 * n);
    L.t = (float*)dalloc(ctx, ps, 4 * n);
    if (l == 0) {
      L.type = ps->type0;
    } else {
      uint8_t* ty = (uint8_t*)dalloc(ctx, ps, n);
      SF_CUDA(cudaMemcpyAsync(ty, types[l].data(), n, cudaMemcpyHostToDevice, ctx->stream));
      L.type = ty;
    }
    SF_CUDA(cudaMemsetAsync(L.y, 0, 4 * n, ctx->stream));
    SF_CUDA(cudaMemsetAsync(L.P, 0, 4 * n, ctx->stream));
    ps->lv.push_back(L);
    const bool can = ((lni - 1) % 2 == 0) && ((lnj - 1) % 2 == 0) && lni >= 5 && lnj >= 5;
    if (!can) break;
    const int cni = (lni - 1) / 2 + 1, cnj = (lnj - 1) / 2 + 1;
    std::vector<uint8_t> tc((size_t)cni * cnj);
    for (int J = 0; J < cnj; J++)
      for (int I = 0; I < cni; I++)
        tc[(size_t)J * cni + I] = node_class(types[l][(size_t)(2 * J) * lni + 2 * I] == NC_FIXED, I, J, cni, cnj);
    types.push_back(tc);
    lni = cni;
    lnj = cnj;
    ldx *= 2;
    ldy *= 2;
  }
  // first level small enough for the single-CTA coarse solve (one mesh, batched solve)
  const int nl = (int)ps->lv.size();
  auto split = [&](int nodes) {
    for (int l = 0; l < nl; l++)
      if ((size_t)ps->lv[l].ni * ps->lv[l].nj <= (size_t)nodes) return l;
    return nl - 1;
  };
  auto desc = [&](int cs, CoarseDesc& D) {
    D.n = nl - cs;
    int off = 0;
    for (int k = 0; k < D.n; k++) {
      const LevelView& L = ps->lv[cs + k];
      D.ni[k] = L.ni;
      D.nj[k] = L.nj;
      D.cx[k] = L.cx;
      D.cy[k] = L.cy;
      D.off[k] = off;
      off += L.ni * L.nj;
    }
    D.total = off;
    const LevelView& Lc = ps->lv[nl - 1];
    D.coarsest_sweeps = std::min(200, std::max(10, std::max(Lc.ni, Lc.nj)));
    D.omega = (float)(2.0 / (1.0 + std::sin(PI / std::max(Lc.ni, Lc.nj))));
    return (size_t)D.total * (4 * sizeof(float) + 1) + 16;
  };
  ps->cs = split(COARSE_NODES);
  ps->coarse_smem = desc(ps->cs, ps->cd);
  ps->cs_b = split(COARSE_NODES_BATCH);
  ps->coarse_smem_b = desc(ps->cs_b, ps->cd_b);
  SF_REQUIRE(ps->coarse_smem <= COARSE_SMEM_MAX && ps->coarse_smem_b <= COARSE_SMEM_MAX, SF_ERR_ARG,
             "mesh not coarsenable to a level that fits in shared memory (use (2^k)m+1 nodes per direction)");
  // the limit is a property of the kernel on the device, shared by every context: always
  // the same bound, so that a context with a smaller coarse end cannot lower it under the
  // launches (and captured graphs) of another
  SF_CUDA(cudaFuncSetAttribute(k_coarse_vcycle, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)COARSE_SMEM_MAX));
  SF_CUDA(cudaEventCreate(&ps->ev0));
  SF_CUDA(cudaEventCreate(&ps->ev1));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  return ps;
}

static inline dim3 grid2(int ni, int nj, dim3 blk) { return dim3((ni + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y); }

static void restrict_P(sf_ctx* ctx, SfPoisson* ps) {
  const dim3 blk(32, 8);
  for (int l = 0; l < ps->cs; l++) {
    k_restrict_P<<<grid2(ps->lv[l + 1].ni, ps->lv[l + 1].nj, blk), blk, 0, ctx->stream>>>(ps->lv[l], ps->lv[l + 1]);
    ctx->launches++;
  }
}

// z = M^-1 r: one V(nu1,nu2)-cycle on level 0 from zero, r = lv[0].r, z -> lv[0].y
// nu red-black sweeps on a level; first = the colour updated first in each sweep
// one tiled level kernel: on levels of a million nodes or more 64 x 32 tiles on the way
// down and 64 x 16 on the way up, 32 x 8 below (shorter per-block chains where the grid is
// too small to fill the GPU)
static void level_down(cudaStream_t s, const LevelView& F, const LevelView& C) {
  if ((size_t)F.ni * F.nj >= (1u << 20))
    // 64x32 tiles on the way down (halo 6: 1.6x the tile's nodes are swept instead of 2.1x
    // for 64x16; 48 registers)
    k_level_down<64, 32><<<dim3((F.ni + 63) / 64, (F.nj + 31) / 32), TILE_NT, 0, s>>>(F, C);
  else
    k_level_down<32, 8><<<dim3((F.ni + 31) / 32, (F.nj + 7) / 8), TILE_NT, 0, s>>>(F, C);
}
static void level_up(cudaStream_t s, const LevelView& F, const LevelView& C) {
  if ((size_t)F.ni * F.nj >= (1u << 20))
    k_level_up<64, 16><<<dim3((F.ni + 63) / 64, (F.nj + 15) / 16), TILE_NT, 0, s>>>(F, C);
  else
    k_level_up<32, 8><<<dim3((F.ni + 31) / 32, (F.nj + 7) / 8), TILE_NT, 0, s>>>(F, C);
}

// Names of the per-kernel timers of the solve (sf_timing_enable): the level kernels per
// level, so that each level's bytes can be divided by its own time.
static const char* level_timer(bool down, int l) {
  static const char* dn[] = {"mg_down_L0", "mg_down_L1", "mg_down_L2", "mg_down_L3", "mg_down_L4", "mg_down_L5",
                             "mg_down_L6", "mg_down_L7"};
  static const char* up[] = {"mg_up_L0", "mg_up_L1", "mg_up_L2", "mg_up_L3", "mg_up_L4", "mg_up_L5",
                             "mg_up_L6", "mg_up_L7"};
  if (l > 7) return down ? "mg_down_L8+" : "mg_up_L8+";
  return down ? dn[l] : up[l];
}

static void vcycle(sf_ctx* ctx, SfPoisson* ps) {
  cudaStream_t s = ctx->stream;
  for (int l = 0; l < ps->cs; l++) {
    TimedScope ts(ctx, level_timer(true, l));
    level_down(s, ps->lv[l], ps->lv[l + 1]);
  }
  {
    TimedScope ts(ctx, "mg_coarse");
    k_coarse_vcycle<<<1, 1024, ps->coarse_smem, s>>>(ps->cd, ps->lv[ps->cs], 2, 2);
  }
  for (int l = ps->cs - 1; l >= 0; l--) {
    TimedScope ts(ctx, level_timer(false, l));
    level_up(s, ps->lv[l], ps->lv[l + 1]);
  }
  ctx->launches += 2 * ps->cs + 1;
}

static void reduce(sf_ctx* ctx, SfPoisson* ps, double* out, int max2) {
  k_reduce_partials<<<1, 256, 0, ctx->stream>>>(ps->partial, ps->red_blocks, out, max2);
  ctx->launches++;
}

// iters steps of flexible PCG on J y = F (F = lv[0].r, overwritten as the CG residual);
// the correction is left in cg_x
// z = M^-1 r on level 0 (r = lv[0].r, z -> lv[0].y): the V-cycle, for an axisymmetric
// mesh between the radius scalings of the row-weighted system
static void precond(sf_ctx* ctx, SfPoisson* ps, int g) {
  if (!ps->axi) {
    vcycle(ctx, ps);
    return;
  }
  k_axi_pre<<<g, 256, 0, ctx->stream>>>(ps->lv[0], ps->axv, ps->axi_keep);
  vcycle(ctx, ps);
  k_axi_post<<<g, 256, 0, ctx->stream>>>(ps->lv[0], ps->axv, ps->axi_keep);
  ctx->launches += 2;
}

static void pcg(sf_ctx* ctx, SfPoisson* ps, int iters, bool coarse) {
  cudaStream_t s = ctx->stream;
  const LevelView& L0 = ps->lv[0];
  const int n = L0.ni * L0.nj;
  const int g = grid_for(n, 256, ctx->num_sms * 8);
  SF_CUDA(cudaMemsetAsync(ps->cg_x, 0, 4 * (size_t)n, s));
  if (coarse) {
    // z0 = e + V(r - J e), e the network's coarse correction of r (cg_p holds r meanwhile;
    // it is first written by the p update below)
    TimedScope ts(ctx, "learned_coarse");
    const float* e = sf_unet_coarse_correction(ctx, L0.r, L0.P, L0.type);
    k_pc_residual<<<g, 256, 0, s>>>(L0, e, ps->cg_p);
    vcycle(ctx, ps);
    k_pc_finish<<<g, 256, 0, s>>>(L0, e, ps->cg_p);
    ctx->launches += 2;
  } else {
    precond(ctx, ps, g);  // z0
  }
  SF_CUDA(cudaMemsetAsync(ps->cg_zo, 0, 4 * (size_t)n, s));
  k_cg_dots<<<ps->red_blocks, RB, 0, s>>>(n, L0.r, L0.y, ps->cg_zo, ps->partial);
  reduce(ctx, ps, ps->sc + SC_RED, 0);
  k_cg_scalars<<<1, 32, 0, s>>>(ps->sc, 0);
  k_cg_pupdate<<<g, 256, 0, s>>>(n, ps->sc, 1, L0.y, ps->cg_p);
  ctx->launches += 3;
  for (int k = 0; k < iters; k++) {
    {
      TimedScope ts(ctx, "cg_matvec");
      if (ps->axi)
        k_cg_matvec_axi<<<ps->red_blocks, RB, 0, s>>>(L0, ps->axv, ps->cg_p, ps->cg_q, ps->partial);
      else
        k_cg_matvec<<<ps->red_blocks, RB, 0, s>>>(L0, ps->cg_p, ps->cg_q, ps->partial);
    }
    reduce(ctx, ps, ps->sc + SC_RED, 0);
    k_cg_scalars<<<1, 32, 0, s>>>(ps->sc, 1);
    k_cg_axpy<<<g, 256, 0, s>>>(n, ps->sc, ps->cg_p, ps->cg_q, ps->cg_x, L0.r, L0.y, ps->cg_zo);
    ctx->launches += 3;
    if (k == iters - 1) break;
    precond(ctx, ps, g);
    k_cg_dots<<<ps->red_blocks, RB, 0, s>>>(n, L0.r, L0.y, ps->cg_zo, ps->partial);
    reduce(ctx, ps, ps->sc + SC_RED, 0);
    k_cg_scalars<<<1, 32, 0, s>>>(ps->sc, 2);
    k_cg_pupdate<<<g, 256, 0, s>>>(n, ps->sc, 0, L0.y, ps->cg_p);
    ctx->launches += 3;
  }
}

// The inner work of one Newton step -- restriction of P, `iters` PCG iterations with
// their V-cycles, phi -= correction -- is ~70 launches of mostly small kernels; it is
// captured once as a CUDA graph and replayed, re-captured when its parameters change.
// With per-kernel timing on, the same launches run directly on the stream, each
// bracketed by its timer's events.
static void newton_step(sf_ctx* ctx, SfPoisson* ps, int iters, double max_step, bool coarse) {
  cudaStream_t s = ctx->stream;
  const int nn = ps->ni * ps->nj;
  if (ctx->timer.on) {
    restrict_P(ctx, ps);
    pcg(ctx, ps, iters, coarse);
    k_update_phi<<<grid_for(nn, 256, ctx->num_sms * 8), 256, 0, s>>>(nn, ps->phi, ps->cg_x, max_step);
    ctx->launches++;
    return;
  }
  const int gi = coarse ? 1 : 0;
  if (!ps->step_graph[gi] || ps->graph_iters[gi] != iters || ps->graph_max_step[gi] != max_step) {
    if (ps->step_graph[gi]) {
      SF_CUDA(cudaGraphExecDestroy(ps->step_graph[gi]));
      ps->step_graph[gi] = nullptr;
    }
    const int64_t l0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    SF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      restrict_P(ctx, ps);
      pcg(ctx, ps, iters, coarse);
      k_update_phi<<<grid_for(nn, 256, ctx->num_sms * 8), 256, 0, s>>>(nn, ps->phi, ps->cg_x, max_step);
      ctx->launches++;
    } catch (...) {
      cudaStreamEndCapture(s, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    SF_CUDA(cudaStreamEndCapture(s, &graph));
    const cudaError_t e = cudaGraphInstantiate(&ps->step_graph[gi], graph, 0);
    cudaGraphDestroy(graph);
    SF_CUDA(e);
    ps->graph_iters[gi] = iters;
    ps->graph_max_step[gi] = max_step;
    ps->graph_launches[gi] = ctx->launches - l0;
    ctx->launches = l0;
  }
  SF_CUDA(cudaGraphLaunch(ps->step_graph[gi], s));
  ctx->launches += ps->graph_launches[gi];
}

void sf_poisson_destroy_internal(sf_ctx* ctx) {
  SfPoisson* ps = ctx->poisson;
  if (!ps) return;
  for (void* p : ps->allocs) cudaFree(p);
  if (ps->ev0) cudaEventDestroy(ps->ev0);
  if (ps->ev1) cudaEventDestroy(ps->ev1);
  for (cudaGraphExec_t g : ps->step_graph)
    if (g) cudaGraphExecDestroy(g);
  delete ps;
  ctx->poisson = nullptr;
}

int sf_poisson_get_field_internal(sf_ctx* ctx, int field, double* out) {
  try {
    SfPoisson* ps = poisson_get(ctx);
    const size_t nn = (size_t)ctx->ni * ctx->nj;
    const double* src = nullptr;
    switch (field) {
      case SF_FIELD_PHI: src = ps->phi; break;
      case SF_FIELD_RHO: src = ps->rho; break;
      case SF_FIELD_EFI: src = ps->efi; break;
      case SF_FIELD_EFJ: src = ps->efj; break;
      case SF_FIELD_NE: src = ps->ne; break;
      default: SF_REQUIRE(false, SF_ERR_ARG, "unknown field selector");
    }
    SF_CUDA(cudaMemcpyAsync(out, src, 8 * nn, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    return SF_OK;
  } catch (const sf::Error& e) {
    ctx->err = e.what();
    return e.code;
  }
}

extern "C" {

int sf_update_rho(sf_ctx* ctx) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null context");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfPoisson* ps = poisson_get(ctx);
  const int nn = ctx->ni * ctx->nj;
  SF_CUDA(cudaMemsetAsync(ps->rho, 0, 8 * (size_t)nn, ctx->stream));
  for (SfSpecies* sp : ctx->species) {
    if (sp->charge == 0) continue;
    k_rho_add<<<grid_for(nn, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(nn, sp->nd, sp->charge, ps->rho);
    ctx->launches++;
  }
  SF_CUDA(cudaGetLastError());
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  ps->rho_set = true;
  SF_API_END(ctx)
}

int sf_set_bc_values(sf_ctx* ctx, const double* bc) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && bc, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfPoisson* ps = poisson_get(ctx);
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  std::copy(bc, bc + nn, ctx->bc_value.begin());
  SF_CUDA(cudaMemcpyAsync(ps->bc, bc, 8 * nn, cudaMemcpyHostToDevice, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  SF_API_END(ctx)
}

int sf_poisson_nl(sf_ctx* ctx, const sf_poisson_params* prm, const double* rho, double* phi, sf_solve_stats* stats) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && prm, SF_ERR_ARG, "null argument");
  SF_REQUIRE(prm->eps > 0 && prm->tol > 0 && prm->max_it > 0, SF_ERR_ARG, "bad solver parameters");
  SF_REQUIRE(prm->linear || (prm->kTe0 > 0 && prm->n0 > 0), SF_ERR_ARG, "Boltzmann electrons need n0 > 0 and kTe0 > 0");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfPoisson* ps = poisson_get(ctx);
  cudaStream_t s = ctx->stream;
  const int nn = ctx->ni * ctx->nj;
  if (rho) {
    SF_CUDA(cudaMemcpyAsync(ps->rho, rho, 8 * (size_t)nn, cudaMemcpyHostToDevice, s));
    ps->rho_set = true;
  }
  SF_REQUIRE(ps->rho_set, SF_ERR_STATE, "no charge density: pass rho or call sf_update_rho");
  if (phi) SF_CUDA(cudaMemcpyAsync(ps->phi, phi, 8 * (size_t)nn, cudaMemcpyHostToDevice, s));
  const int g = grid_for(nn, 256, ctx->num_sms * 8);
  k_build_b0<<<g, 256, 0, s>>>(nn, ps->rho, ps->bc, ps->type0, 1.0 / prm->eps, ps->b0);
  k_fix_phi<<<g, 256, 0, s>>>(nn, ps->phi, ps->bc, ps->type0);  // fixed rows exact from the start
  ctx->launches += 2;
  ps->prm = *prm;
  ps->have_prm = true;
  NlArgs a;
  a.ni = ctx->ni;
  a.nj = ctx->nj;
  a.dx = ctx->dh[0];
  a.dy = ctx->dh[1];
  a.cx = 1.0 / (a.dx * a.dx);
  a.cy = 1.0 / (a.dy * a.dy);
  a.C_n0 = QE / prm->eps * prm->n0;
  a.inv_kTe = prm->linear ? 0.0 : 1.0 / prm->kTe0;
  a.phi0 = prm->phi0;
  a.linear = prm->linear ? 1 : 0;
  a.fp64_exp = ps->fp64_exp ? 1 : 0;
  a.axi = ps->axi;
  a.r0 = ps->r0;
  a.dr = ps->dr;
  SF_REQUIRE(!ps->axi || prm->use_learned == 0, SF_ERR_ARG, "the learned modes take XY meshes");
  // the radius-scaled preconditioner is weaker near the axis: more PCG steps per Newton step
  const int iters = prm->cycles > 0 ? prm->cycles : (ps->axi ? 6 : 4);
  SF_CUDA(cudaEventRecord(ps->ev0, s));
  double h[3];
  // FP64 residual of the current phi into level 0 (F, P) and its norms.  The FP32
  // exponential's error bound is checked against the tolerance: its worst node adds at
  // most h[2] / sqrt(nn) to ||R||_2 / N; past 1 % of tol the solve continues in FP64.
  auto residual = [&](double* r2, double* rinf) {
    for (;;) {
      {
        TimedScope ts(ctx, "nl_residual");
        k_nl_residual<<<ps->red_blocks, RB, 0, s>>>(a, ps->phi, ps->b0, ps->type0, ps->lv[0].r, ps->lv[0].P,
                                                    ps->partial);
      }
      k_reduce_partials3<<<1, 256, 0, s>>>(ps->partial, ps->red_blocks, ps->red);
      ctx->launches += 2;
      SF_CUDA(cudaMemcpyAsync(h, ps->red, 24, cudaMemcpyDeviceToHost, s));
      SF_CUDA(cudaStreamSynchronize(s));
      if (!a.fp64_exp && h[2] / std::sqrt((double)nn) > 0.01 * prm->tol) {
        a.fp64_exp = 1;
        continue;
      }
      *r2 = std::sqrt(h[0]) / nn;
      *rinf = h[1];
      return;
    }
  };
  // learned warm start (inside the timed region): phi <- phi_prev + U-Net prediction of
  // the change, kept only if its FP64 residual is below that of phi_prev itself
  double res = 0, res_inf = 0, res0 = -1;
  if (prm->use_learned == 1 && !phi && ctx->unet) {
    double r_prev, rinf_prev;
    residual(&r_prev, &rinf_prev);
    if (sf_unet_warm_start(ctx, ps->phi, ps->rho, ps->bc, ps->type0)) {
      residual(&res, &res_inf);
      if (!(res < r_prev)) {
        // back to the previous potential, with this solve's Dirichlet values (the inner
        // system is symmetric only while the fixed rows are exact)
        sf_unet_reject(ctx, ps->phi);
        k_fix_phi<<<g, 256, 0, s>>>(nn, ps->phi, ps->bc, ps->type0);
        ctx->launches++;
        residual(&res, &res_inf);
      }
    } else {
      res = r_prev;
      res_inf = rinf_prev;
    }
    res0 = res;
  }
  // coarse-correction mode (use_learned = 2): once trained, the network corrects the first
  // preconditioner application of the solve's first Newton step -- the residual it is
  // trained on (later steps' residuals are orders of magnitude smaller and dominated by
  // the particle noise of rho); every converged solve in this mode trains it on its own
  // first residual
  const bool coarse_mode = prm->use_learned == 2 && ctx->unet;
  const bool coarse = coarse_mode && sf_unet_coarse_ready(ctx);
  int it = 0, vcount = 0;
  bool conv = false, diverged = false;
  for (it = 0; it <= prm->max_it; it++) {
    if (it > 0 || res0 < 0) residual(&res, &res_inf);
    if (res0 < 0) res0 = res;
    if (!std::isfinite(res)) {
      diverged = true;
      break;
    }
    if (res < prm->tol) {
      conv = true;
      break;
    }
    if (it == prm->max_it) break;
    if (it == 0 && coarse_mode) sf_unet_coarse_start(ctx, ps->lv[0].r, ps->lv[0].P, ps->phi);
    newton_step(ctx, ps, iters, prm->linear ? 1e300 : 10.0 * prm->kTe0, coarse && it == 0);
    vcount += iters;
  }
  ps->fp64_exp = a.fp64_exp != 0;
  SF_CUDA(cudaEventRecord(ps->ev1, s));
  SF_CUDA(cudaEventSynchronize(ps->ev1));
  float ms = 0;
  SF_CUDA(cudaEventElapsedTime(&ms, ps->ev0, ps->ev1));
  SF_CUDA(cudaGetLastError());
  // every converged solve is a training pair for the warm-start network (outside the
  // timed region; its cost is reported by sf_unet_stats)
  if (conv && coarse_mode) sf_unet_coarse_train(ctx, ps->phi, ps->type0);
  else if (conv && ctx->unet) sf_unet_after_solve(ctx, ps->phi, ps->rho, ps->bc, ps->type0, prm->eps);
  if (phi) {
    SF_CUDA(cudaMemcpyAsync(phi, ps->phi, 8 * (size_t)nn, cudaMemcpyDeviceToHost, s));
    SF_CUDA(cudaStreamSynchronize(s));
  }
  if (stats) {
    stats->newton_it = it;
    stats->vcycles = vcount;
    stats->residual = res;
    stats->residual_inf = res_inf;
    stats->initial_residual = res0;
    stats->ms = ms;
  }
  SF_REQUIRE(!diverged, SF_ERR_DIVERGED, "Solver diverged (non-finite residual)");
  SF_REQUIRE(conv, SF_ERR_NOT_CONVERGED, "Poisson solve did not reach the residual tolerance");
  SF_API_END(ctx)
}

int sf_efield(sf_ctx* ctx, double* efi, double* efj) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null context");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfPoisson* ps = poisson_get(ctx);
  const int nn = ctx->ni * ctx->nj;
  k_efield<<<grid_for(nn, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      ctx->ni, ctx->nj, 1.0 / ctx->dh[0], 1.0 / ctx->dh[1], ps->phi, ps->efi, ps->efj, ctx->E);
  ctx->launches++;
  SF_CUDA(cudaGetLastError());
  if (efi) SF_CUDA(cudaMemcpyAsync(efi, ps->efi, 8 * (size_t)nn, cudaMemcpyDeviceToHost, ctx->stream));
  if (efj) SF_CUDA(cudaMemcpyAsync(efj, ps->efj, 8 * (size_t)nn, cudaMemcpyDeviceToHost, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->efield_set = true;
  SF_API_END(ctx)
}

int sf_boltzmann(sf_ctx* ctx, double* ne) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null context");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfPoisson* ps = poisson_get(ctx);
  SF_REQUIRE(ps->have_prm && !ps->prm.linear, SF_ERR_STATE, "no Boltzmann parameters: run sf_poisson_nl first");
  const int nn = ctx->ni * ctx->nj;
  k_boltzmann<<<grid_for(nn, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(nn, ps->phi, ps->prm.n0,
                                                                           1.0 / ps->prm.kTe0, ps->prm.phi0, ps->ne);
  ctx->launches++;
  SF_CUDA(cudaGetLastError());
  if (ne) SF_CUDA(cudaMemcpyAsync(ne, ps->ne, 8 * (size_t)nn, cudaMemcpyDeviceToHost, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  SF_API_END(ctx)
}

}  // extern "C"

// ------------------------------------------------------------------------------------
// Batched field phase: rho, the nonlinear solve and E of many contexts (sf_batch) with
// one launch per stage for all of them.  Every stage runs the per-node and per-block
// bodies of the single-context kernels on each instance's own buffers, with the same
// reduction partition, so every instance gets the potential its own sf_poisson_nl would
// give, bit for bit.  Convergence is decided per instance on the device; the host reads
// one count per Newton round for the whole batch.  After every check the instances still
// iterating are listed with the prefixes of their blocks, and the stage kernels loop over
// those blocks only, so that the late rounds of a few slow instances cost little.
// ------------------------------------------------------------------------------------
namespace {

constexpr int BP_MAX_SPECIES = 8;
constexpr int ET = 256;  // nodes per block of the elementwise and level kernels

struct BPInst {
  int ni, nj, nn, red_blocks;
  double inv_dx, inv_dy;
  NlArgs nl;  // mesh part of the residual arguments (the step's parameters are added per launch)
  double *phi, *b0, *rho, *efi, *efj, *partial, *red, *sc;
  const double* bc;
  const uint8_t* type0;
  float4* E;
  float *cg_x, *cg_p, *cg_q, *cg_zo;
  int nspecies;
  const double* nd[BP_MAX_SPECIES];
  double q[BP_MAX_SPECIES];
  int cs;
  LevelView lv[MAX_LEVELS];
  CoarseDesc cd;
  // state of the current step
  int iters;     // PCG iterations per Newton step
  int fp64_exp;  // sticky, as SfPoisson::fp64_exp
  int live;      // still iterating (after a check: a Newton step is taken in this round)
  int run;       // a Newton step is taken in this round
  int redo;      // the residual is evaluated again with the FP64 exponential
  int it, vcount, status;  // status: 0 running, 1 converged, 2 not converged, 3 diverged
  double res, res_inf, res0;
};

struct BPParams {
  double C_n0, inv_kTe, phi0, inv_eps, tol, max_step;
  int linear, max_it;
};

struct BPStat {
  int status, it, vcount, fp64_exp;
  double res, res_inf, res0;
};

// The blocks of one launch kind over the live instances: list[0..*cnt) their ids,
// start[k] the first block of list[k], *total all blocks of the kind.
struct BPWork {
  const int* list;
  const int* cnt;
  const int* start;
  const int* total;
};

enum { BP_LIVE = 0, BP_REDO = 1, BP_RUN = 2 };

__device__ __forceinline__ bool bp_part(const BPInst& I, int mode, int kmin) {
  if (mode == BP_LIVE) return I.live != 0;
  if (mode == BP_REDO) return I.redo != 0;
  return I.run != 0 && I.iters > kmin;
}

// entry owning block b: start[k] <= b < start[k + 1]
__device__ __forceinline__ int bp_find(const int* __restrict__ start, int n, int b) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Exclusive prefix of val(0..n-1) into out[0..n] (out[n] = total) by one block whose size
// is a multiple of 32; val(i) is called once per i
template <typename F>
__device__ void bp_prefix(int n, F val, int* __restrict__ out) {
  __shared__ int wsum[32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < n ? val(i) : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = lane < nwarps ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    const int before = carry + (warp > 0 ? wsum[warp - 1] : 0) + x - v;
    if (i < n) out[i] = before;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
  __syncthreads();
}

// The live instances (act_list, *act_cnt) and, for every kind k, the prefix of their
// blocks (act_start + k (n + 1)) and its total (act_total[k]).  tab + koff[k] is the
// static block prefix of kind k over all instances.  The list follows order[] (the
// instances by decreasing coarse-cycle size: the longest single-CTA cycles start first).
// One block.
__global__ void __launch_bounds__(1024) kb_compact(const BPInst* I, int n, const int* __restrict__ order,
                                                   const int* __restrict__ tab, const int* __restrict__ koff,
                                                   int nkinds, int* act_pos, int* act_list, int* act_cnt,
                                                   int* act_start, int* act_total) {
  bp_prefix(n, [&](int q) { return I[order[q]].live ? 1 : 0; }, act_pos);
  for (int q = threadIdx.x; q < n; q += blockDim.x)
    if (I[order[q]].live) act_list[act_pos[q]] = order[q];
  const int cnt = act_pos[n];
  if (threadIdx.x == 0) *act_cnt = cnt;
  __syncthreads();
  for (int k = 0; k < nkinds; k++) {
    const int* t = tab + koff[k];
    int* st = act_start + k * (n + 1);
    bp_prefix(cnt, [&](int q) { const int i = act_list[q]; return t[i + 1] - t[i]; }, st);
    if (threadIdx.x == 0) act_total[k] = st[cnt];
  }
}

__global__ void kb_init(BPInst* I, int n, const int* __restrict__ iters) {
  // iters[0..n): PCG iterations per Newton step, iters[n..2n): the sticky FP64 choice
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  BPInst& s = I[i];
  s.iters = iters[i];
  s.fp64_exp = iters[n + i];
  s.live = 1;
  s.run = 0;
  s.redo = 0;
  s.it = 0;
  s.vcount = 0;
  s.status = 0;
  s.res = s.res_inf = 0.0;
  s.res0 = -1.0;
}

// rho = sum q nd (sf_update_rho), b0 (k_build_b0), fixed rows of phi (k_fix_phi); all instances
__global__ void kb_rho_b0(BPInst* I, int n, const int* __restrict__ start, const BPParams* __restrict__ pr) {
  const int i = bp_find(start, n, blockIdx.x);
  const BPInst& s = I[i];
  const int u = (blockIdx.x - start[i]) * ET + threadIdx.x;
  if (u >= s.nn) return;
  double r = 0.0;
  for (int k = 0; k < s.nspecies; k++) r = rho_add(r, s.q[k], s.nd[k][u]);
  s.rho[u] = r;
  const uint8_t t = s.type0[u];
  s.b0[u] = b0_value(t, s.bc[u], r, pr->inv_eps);
  if (t == NC_FIXED) s.phi[u] = s.bc[u];
}

__global__ void kb_efield(BPInst* I, int n, const int* __restrict__ start) {
  const int i = bp_find(start, n, blockIdx.x);
  const BPInst& s = I[i];
  const int u = (blockIdx.x - start[i]) * ET + threadIdx.x;
  if (u < s.nn) efield_node(u, s.ni, s.nj, s.inv_dx, s.inv_dy, s.phi, s.efi, s.efj, s.E);
}

__global__ void __launch_bounds__(RB) kb_nl_residual(BPInst* I, BPWork w, const BPParams* __restrict__ pr, int mode) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, mode, 0)) continue;
    NlArgs a = s.nl;
    a.C_n0 = pr->C_n0;
    a.inv_kTe = pr->inv_kTe;
    a.phi0 = pr->phi0;
    a.linear = pr->linear;
    a.fp64_exp = s.fp64_exp;
    nl_residual_body(a, s.phi, s.b0, s.type0, s.lv[0].r, s.lv[0].P, s.partial, b - w.start[k], s.red_blocks);
    __syncthreads();  // the block sums' shared memory is used again
  }
}

__global__ void kb_reduce3(BPInst* I, int mode) {
  const BPInst& s = I[blockIdx.x];
  if (!bp_part(s, mode, 0)) return;
  reduce3_body(s.partial, s.red_blocks, s.red);
}

// the FP32 exponential's error bound against the tolerance (the residual lambda of sf_poisson_nl)
__global__ void kb_check_exp(BPInst* I, int n, const BPParams* __restrict__ pr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  BPInst& s = I[i];
  s.redo = 0;
  if (s.live && !s.fp64_exp && s.red[2] / sqrt((double)s.nn) > 0.01 * pr->tol) {
    s.fp64_exp = 1;
    s.redo = 1;
  }
}

// one check of the Newton loop of sf_poisson_nl per live instance; run_count counts the
// instances that take a step in this round (they stay live, the others leave)
__global__ void kb_newton_control(BPInst* I, int n, const BPParams* __restrict__ pr, int* run_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  BPInst& s = I[i];
  s.run = 0;
  if (!s.live) return;
  const double res = sqrt(s.red[0]) / s.nn;
  s.res = res;
  s.res_inf = s.red[1];
  if (s.res0 < 0) s.res0 = res;
  if (!isfinite(res)) {
    s.status = 3;
  } else if (res < pr->tol) {
    s.status = 1;
  } else if (s.it == pr->max_it) {
    s.status = 2;
  } else {
    s.run = 1;
    s.it++;
    s.vcount += s.iters;
    atomicAdd(run_count, 1);
    return;
  }
  s.live = 0;
}

// End of one Newton round of the batched solve, inside the WHILE node of the field-phase
// graph: another round runs while some instance took a Newton step in this one (an
// instance stops stepping once it converges, fails or reaches max_it, so the loop ends
// after at most max_it + 1 rounds; the count is a second bound).
__global__ void kb_round_done(const int* __restrict__ run, int* rounds, const BPParams* __restrict__ pr,
                              cudaGraphConditionalHandle loop) {
  const int k = ++*rounds;
  cudaGraphSetConditional(loop, (*run > 0 && k <= pr->max_it) ? 1u : 0u);
}

// level kernels: grid level l of the live instances with l < cs
__global__ void kb_restrict_P(BPInst* I, BPWork w, int l, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const LevelView& F = s.lv[l];
    const LevelView& Cl = s.lv[l + 1];
    const int uc = (b - w.start[k]) * ET + threadIdx.x;
    if (uc >= Cl.ni * Cl.nj) continue;
    const int J = uc / Cl.ni, Ii = uc - J * Cl.ni;
    Cl.P[uc] = F.P[(2 * J) * F.ni + 2 * Ii];
  }
}

__global__ void kb_zero_y(BPInst* I, BPWork w, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const int u = (b - w.start[k]) * ET + threadIdx.x;
    if (u < s.nn) s.lv[0].y[u] = 0.f;
  }
}

__global__ void kb_smooth(BPInst* I, BPWork w, int l, int color, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const LevelView& L = s.lv[l];
    const int hw = (L.ni + 1) / 2;
    const int v = (b - w.start[k]) * ET + threadIdx.x;
    const int j = v / hw;
    if (j >= L.nj) continue;
    const int ii = 2 * (v - j * hw) + ((j + color) & 1);
    if (ii >= L.ni) continue;
    const int u = j * L.ni + ii;
    L.y[u] = gs_value(L.type[u], L.y, L.r[u], L.P[u], u, L.ni, L.cx, L.cy);
  }
}

__global__ void kb_resid(BPInst* I, BPWork w, int l, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const LevelView& L = s.lv[l];
    const int u = (b - w.start[k]) * ET + threadIdx.x;
    if (u >= L.ni * L.nj) continue;
    L.t[u] = L.r[u] - apply_J(L.type[u], L.y, L.P[u], u, L.ni, L.cx, L.cy);
  }
}

__global__ void kb_restrict(BPInst* I, BPWork w, int l, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const LevelView& F = s.lv[l];
    const LevelView& Cl = s.lv[l + 1];
    const int uc = (b - w.start[k]) * ET + threadIdx.x;
    if (uc >= Cl.ni * Cl.nj) continue;
    const int J = uc / Cl.ni, Ii = uc - J * Cl.ni;
    Cl.r[uc] = restrict_value(F.t, Cl.type[uc], Ii, J, F.ni, Cl.ni, Cl.nj);
    Cl.y[uc] = 0.f;
  }
}

__global__ void kb_prolong(BPInst* I, BPWork w, int l, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const LevelView& F = s.lv[l];
    const LevelView& Cl = s.lv[l + 1];
    const int u = (b - w.start[k]) * ET + threadIdx.x;
    if (u >= F.ni * F.nj) continue;
    if (F.type[u] == NC_FIXED) continue;
    const int j = u / F.ni, ii = u - j * F.ni;
    F.y[u] += prolong_value(Cl.y, ii, j, Cl.ni);
  }
}

// one CTA per live instance at a time (the single-CTA end of the V-cycle)
__global__ void __launch_bounds__(1024, 1) kb_coarse_vcycle(BPInst* I, const int* __restrict__ list,
                                                         const int* __restrict__ cnt, int nu1, int nu2, int kmin) {
  const int c = *cnt;
  for (int k = blockIdx.x; k < c; k += gridDim.x) {
    const BPInst& s = I[list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    coarse_vcycle_body(s.cd, s.lv[s.cs], nu1, nu2);
    __syncthreads();  // the shared arrays are used again
  }
}

// fine-level PCG stages
__global__ void kb_zero_cg(BPInst* I, BPWork w, int which, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const int u = (b - w.start[k]) * ET + threadIdx.x;
    if (u < s.nn) (which == 0 ? s.cg_x : s.cg_zo)[u] = 0.f;
  }
}

__global__ void __launch_bounds__(RB) kb_cg_dots(BPInst* I, BPWork w, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    cg_dots_body(s.nn, s.lv[0].r, s.lv[0].y, s.cg_zo, s.partial, b - w.start[k], s.red_blocks);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(RB) kb_cg_matvec(BPInst* I, BPWork w, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    cg_matvec_body(s.lv[0], s.cg_p, s.cg_q, s.partial, b - w.start[k], s.red_blocks);
    __syncthreads();
  }
}

__global__ void kb_reduce2(BPInst* I, int kmin) {
  const BPInst& s = I[blockIdx.x];
  if (!bp_part(s, BP_RUN, kmin)) return;
  reduce2_body(s.partial, s.red_blocks, s.sc + SC_RED, 0);
}

__global__ void kb_cg_scalars(BPInst* I, int n, int stage, int kmin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BPInst& s = I[i];
  if (!bp_part(s, BP_RUN, kmin)) return;
  cg_scalars_body(s.sc, stage);
}

__global__ void kb_cg_axpy(BPInst* I, BPWork w, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const int u = (b - w.start[k]) * ET + threadIdx.x;
    if (u < s.nn) cg_axpy_node(u, (float)s.sc[SC_ALPHA], s.cg_p, s.cg_q, s.cg_x, s.lv[0].r, s.lv[0].y, s.cg_zo);
  }
}

__global__ void kb_cg_pupdate(BPInst* I, BPWork w, int first, int kmin) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, kmin)) continue;
    const int u = (b - w.start[k]) * ET + threadIdx.x;
    if (u < s.nn) cg_pupdate_node(u, first, first ? 0.f : (float)s.sc[SC_BETA], s.lv[0].y, s.cg_p);
  }
}

__global__ void kb_update_phi(BPInst* I, BPWork w, const BPParams* __restrict__ pr) {
  const int tot = *w.total, cnt = *w.cnt;
  for (int b = blockIdx.x; b < tot; b += gridDim.x) {
    const int k = bp_find(w.start, cnt, b);
    const BPInst& s = I[w.list[k]];
    if (!bp_part(s, BP_RUN, 0)) continue;
    const int u = (b - w.start[k]) * ET + threadIdx.x;
    if (u < s.nn) update_phi_node(u, s.phi, s.cg_x, pr->max_step);
  }
}

__global__ void kb_collect(const BPInst* I, int n, BPStat* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BPInst& s = I[i];
  out[i] = BPStat{s.status, s.it, s.vcount, s.fp64_exp, s.res, s.res_inf, s.res0};
}

}  // namespace

namespace sf {

struct BatchPoisson {
  int n = 0, num_sms = 0;
  std::vector<sf_ctx*> ctx;
  std::vector<int> nspecies;  // charged species per context when the table was built
  BPInst* d_inst = nullptr;
  int* d_tab = nullptr;   // static block prefixes of every kind, n + 1 each
  int* d_koff = nullptr;  // offset of each kind's prefix in d_tab
  int* d_order = nullptr;  // instances by decreasing coarse-cycle size
  int* d_iters = nullptr;
  int* d_run = nullptr;
  int* d_rounds = nullptr;  // Newton rounds of the current field phase
  BPParams* d_prm = nullptr;
  BPStat* d_stat = nullptr;
  // the live list and its per-kind prefixes
  int *d_act_pos = nullptr, *d_act_list = nullptr, *d_act_cnt = nullptr, *d_act_start = nullptr,
      *d_act_total = nullptr;
  // kinds: 0 fine level, 1 reduction blocks, 2 level-0 zero fill (cs > 0), then per grid
  // level l: 3 + 3 l the level, 4 + 3 l the next coarser level, 5 + 3 l one colour
  int nkinds = 0;
  std::vector<int> koff, ktot;  // static offset in d_tab and total blocks per kind
  int max_cs = 0;
  size_t coarse_smem = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t body_stream = nullptr;  // captures the Newton round into the WHILE node's body
  std::vector<std::pair<int, cudaGraphExec_t>> graphs;  // field phase by max PCG iterations
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

enum { BK_FINE = 0, BK_RED = 1, BK_ZERO = 2 };
static inline int bk_lvl(int l) { return 3 + 3 * l; }
static inline int bk_lvlc(int l) { return 4 + 3 * l; }
static inline int bk_half(int l) { return 5 + 3 * l; }

static BPWork bp_work(const BatchPoisson* bp, int kind) {
  return BPWork{bp->d_act_list, bp->d_act_cnt, bp->d_act_start + kind * (bp->n + 1), bp->d_act_total + kind};
}

// grid of a stage kernel: the kind's blocks over all instances, at most 8 per SM (the
// kernels loop over the live blocks)
static int bp_grid(const BatchPoisson* bp, int kind) {
  return std::max(1, std::min(bp->ktot[kind], bp->num_sms * 8));
}

static void bp_compact(BatchPoisson* bp, cudaStream_t s) {
  kb_compact<<<1, 1024, 0, s>>>(bp->d_inst, bp->n, bp->d_order, bp->d_tab, bp->d_koff, bp->nkinds,
                                bp->d_act_pos, bp->d_act_list, bp->d_act_cnt, bp->d_act_start, bp->d_act_total);
}

static void bp_vcycle(BatchPoisson* bp, cudaStream_t s, int kmin) {
  BPInst* I = bp->d_inst;
  if (bp->ktot[BK_ZERO] > 0) kb_zero_y<<<bp_grid(bp, BK_ZERO), ET, 0, s>>>(I, bp_work(bp, BK_ZERO), kmin);
  for (int l = 0; l < bp->max_cs; l++) {
    const BPWork half = bp_work(bp, bk_half(l));
    const int gh = bp_grid(bp, bk_half(l));
    for (int k = 0; k < 2; k++) {
      kb_smooth<<<gh, ET, 0, s>>>(I, half, l, 0, kmin);
      kb_smooth<<<gh, ET, 0, s>>>(I, half, l, 1, kmin);
    }
    kb_resid<<<bp_grid(bp, bk_lvl(l)), ET, 0, s>>>(I, bp_work(bp, bk_lvl(l)), l, kmin);
    kb_restrict<<<bp_grid(bp, bk_lvlc(l)), ET, 0, s>>>(I, bp_work(bp, bk_lvlc(l)), l, kmin);
  }
  kb_coarse_vcycle<<<bp->n, 1024, bp->coarse_smem, s>>>(I, bp->d_act_list, bp->d_act_cnt, 2, 2, kmin);
  for (int l = bp->max_cs - 1; l >= 0; l--) {
    kb_prolong<<<bp_grid(bp, bk_lvl(l)), ET, 0, s>>>(I, bp_work(bp, bk_lvl(l)), l, kmin);
    const BPWork half = bp_work(bp, bk_half(l));
    const int gh = bp_grid(bp, bk_half(l));
    for (int k = 0; k < 2; k++) {
      kb_smooth<<<gh, ET, 0, s>>>(I, half, l, 1, kmin);
      kb_smooth<<<gh, ET, 0, s>>>(I, half, l, 0, kmin);
    }
  }
}

// One Newton round of every live instance: the residual (again in FP64 where the FP32
// exponential's bound fails), the convergence check, the list of the instances going on,
// and their Newton step: restriction of P, PCG with the instance's iterations, phi update.
static void bp_round(BatchPoisson* bp, cudaStream_t s, int max_iters) {
  const int n = bp->n;
  BPInst* I = bp->d_inst;
  const BPWork fine = bp_work(bp, BK_FINE), red = bp_work(bp, BK_RED);
  const int gf = bp_grid(bp, BK_FINE), gr = bp_grid(bp, BK_RED);
  const int tb = 128, tg = (n + tb - 1) / tb;
  SF_CUDA(cudaMemsetAsync(bp->d_run, 0, sizeof(int), s));
  kb_nl_residual<<<gr, RB, 0, s>>>(I, red, bp->d_prm, BP_LIVE);
  kb_reduce3<<<n, 256, 0, s>>>(I, BP_LIVE);
  kb_check_exp<<<tg, tb, 0, s>>>(I, n, bp->d_prm);
  kb_nl_residual<<<gr, RB, 0, s>>>(I, red, bp->d_prm, BP_REDO);
  kb_reduce3<<<n, 256, 0, s>>>(I, BP_REDO);
  kb_newton_control<<<tg, tb, 0, s>>>(I, n, bp->d_prm, bp->d_run);
  bp_compact(bp, s);
  for (int l = 0; l < bp->max_cs; l++)
    kb_restrict_P<<<bp_grid(bp, bk_lvlc(l)), ET, 0, s>>>(I, bp_work(bp, bk_lvlc(l)), l, 0);
  kb_zero_cg<<<gf, ET, 0, s>>>(I, fine, 0, 0);
  bp_vcycle(bp, s, 0);
  kb_zero_cg<<<gf, ET, 0, s>>>(I, fine, 1, 0);
  kb_cg_dots<<<gr, RB, 0, s>>>(I, red, 0);
  kb_reduce2<<<n, 256, 0, s>>>(I, 0);
  kb_cg_scalars<<<tg, tb, 0, s>>>(I, n, 0, 0);
  kb_cg_pupdate<<<gf, ET, 0, s>>>(I, fine, 1, 0);
  for (int k = 0; k < max_iters; k++) {
    kb_cg_matvec<<<gr, RB, 0, s>>>(I, red, k);
    kb_reduce2<<<n, 256, 0, s>>>(I, k);
    kb_cg_scalars<<<tg, tb, 0, s>>>(I, n, 1, k);
    kb_cg_axpy<<<gf, ET, 0, s>>>(I, fine, k);
    if (k == max_iters - 1) break;
    bp_vcycle(bp, s, k + 1);
    kb_cg_dots<<<gr, RB, 0, s>>>(I, red, k + 1);
    kb_reduce2<<<n, 256, 0, s>>>(I, k + 1);
    kb_cg_scalars<<<tg, tb, 0, s>>>(I, n, 2, k + 1);
    kb_cg_pupdate<<<gf, ET, 0, s>>>(I, fine, 0, k + 1);
  }
  kb_update_phi<<<gf, ET, 0, s>>>(I, fine, bp->d_prm);
  SF_CUDA(cudaGetLastError());
}

template <typename F>
static void bp_table(std::vector<int>& tab, int n, F blocks, int& off, int& tot) {
  off = (int)tab.size();
  int acc = 0;
  for (int i = 0; i < n; i++) {
    tab.push_back(acc);
    acc += blocks(i);
  }
  tab.push_back(acc);
  tot = acc;
}

// The whole field phase as one CUDA graph: the instances' start state, rho and b0, the
// live list, then a WHILE node whose body is one Newton round of every live instance
// (bp_round) followed by kb_round_done, which decides on the device whether another round
// runs; then E and the per-instance results.  The host reads nothing until the phase is
// done.  Graphs are kept per number of PCG iterations (the round's launch sequence).
static cudaGraphExec_t bp_graph(BatchPoisson* bp, int max_iters) {
  for (auto& g : bp->graphs)
    if (g.first == max_iters) return g.second;
  cudaStream_t s = bp->stream;
  const int n = bp->n, tg = (n + 127) / 128;
  cudaGraph_t graph = nullptr;
  SF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaGraphConditionalHandle loop{};
  cudaGraph_t body = nullptr;
  try {
    kb_init<<<tg, 128, 0, s>>>(bp->d_inst, n, bp->d_iters);
    kb_rho_b0<<<bp->ktot[BK_FINE], ET, 0, s>>>(bp->d_inst, n, bp->d_tab + bp->koff[BK_FINE], bp->d_prm);
    bp_compact(bp, s);  // every instance is live
    SF_CUDA(cudaMemsetAsync(bp->d_rounds, 0, sizeof(int), s));
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    SF_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &ndeps));
    SF_CUDA(cudaGraphConditionalHandleCreate(&loop, g, 1u, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    SF_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
    body = cp.conditional.phGraph_out[0];
    SF_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    kb_efield<<<bp->ktot[BK_FINE], ET, 0, s>>>(bp->d_inst, n, bp->d_tab + bp->koff[BK_FINE]);
    kb_collect<<<tg, 128, 0, s>>>(bp->d_inst, n, bp->d_stat);
    SF_CUDA(cudaGetLastError());
  } catch (...) {
    cudaStreamEndCapture(s, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  SF_CUDA(cudaStreamEndCapture(s, &graph));
  try {
    SF_CUDA(cudaStreamBeginCaptureToGraph(bp->body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    try {
      bp_round(bp, bp->body_stream, max_iters);
      kb_round_done<<<1, 1, 0, bp->body_stream>>>(bp->d_run, bp->d_rounds, bp->d_prm, loop);
      SF_CUDA(cudaGetLastError());
    } catch (...) {
      cudaGraph_t b2 = nullptr;
      cudaStreamEndCapture(bp->body_stream, &b2);
      throw;
    }
    SF_CUDA(cudaStreamEndCapture(bp->body_stream, &body));
  } catch (...) {
    cudaGraphDestroy(graph);
    throw;
  }
  cudaGraphExec_t ex = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&ex, graph, 0);
  cudaGraphDestroy(graph);
  SF_CUDA(e);
  bp->graphs.push_back({max_iters, ex});
  return ex;
}

static int charged_species(const sf_ctx* c) {
  int k = 0;
  for (const SfSpecies* sp : c->species)
    if (sp->charge != 0) k++;
  return k;
}

// the instance table from the contexts' current state
static void bp_fill(BatchPoisson* bp) {
  std::vector<BPInst> h(bp->n);
  bp->nspecies.assign(bp->n, 0);
  for (int i = 0; i < bp->n; i++) {
    sf_ctx* c = bp->ctx[i];
    SfPoisson* ps = poisson_get(c);
    BPInst& s = h[i];
    std::memset(&s, 0, sizeof(s));
    s.ni = c->ni;
    s.nj = c->nj;
    s.nn = c->ni * c->nj;
    s.red_blocks = ps->red_blocks;
    s.inv_dx = 1.0 / c->dh[0];
    s.inv_dy = 1.0 / c->dh[1];
    s.nl.ni = c->ni;
    s.nl.nj = c->nj;
    s.nl.dx = c->dh[0];
    s.nl.dy = c->dh[1];
    s.nl.cx = 1.0 / (s.nl.dx * s.nl.dx);
    s.nl.cy = 1.0 / (s.nl.dy * s.nl.dy);
    s.phi = ps->phi;
    s.b0 = ps->b0;
    s.rho = ps->rho;
    s.efi = ps->efi;
    s.efj = ps->efj;
    s.partial = ps->partial;
    s.red = ps->red;
    s.sc = ps->sc;
    s.bc = ps->bc;
    s.type0 = ps->type0;
    s.E = c->E;
    s.cg_x = ps->cg_x;
    s.cg_p = ps->cg_p;
    s.cg_q = ps->cg_q;
    s.cg_zo = ps->cg_zo;
    for (const SfSpecies* sp : c->species) {
      if (sp->charge == 0) continue;
      SF_REQUIRE(s.nspecies < BP_MAX_SPECIES, SF_ERR_ARG, "too many charged species for the batched solve");
      s.nd[s.nspecies] = sp->nd;
      s.q[s.nspecies] = sp->charge;
      s.nspecies++;
    }
    bp->nspecies[i] = s.nspecies;
    s.cs = ps->cs_b;
    for (size_t l = 0; l < ps->lv.size(); l++) s.lv[l] = ps->lv[l];
    s.cd = ps->cd_b;
    s.fp64_exp = ps->fp64_exp ? 1 : 0;
  }
  copy_wait(bp->d_inst, h.data(), sizeof(BPInst) * bp->n, cudaMemcpyHostToDevice, bp->stream);
}

BatchPoisson* batch_poisson_create(sf_ctx* const* ctxs, int n, int num_sms, cudaStream_t stream) {
  auto* bp = new BatchPoisson();
  try {
    bp->n = n;
    bp->num_sms = num_sms;
    bp->stream = stream;
    bp->ctx.assign(ctxs, ctxs + n);
    std::vector<SfPoisson*> ps(n);
    for (int i = 0; i < n; i++) {
      SF_REQUIRE(ctxs[i]->domain == SF_DOMAIN_XY, SF_ERR_ARG, "the batched solve takes XY meshes");
      ps[i] = poisson_get(ctxs[i]);
      bp->max_cs = std::max(bp->max_cs, ps[i]->cs_b);
      bp->coarse_smem = std::max(bp->coarse_smem, ps[i]->coarse_smem_b);
    }
    std::vector<int> tab;
    bp->nkinds = 3 + 3 * bp->max_cs;
    bp->koff.assign(bp->nkinds, 0);
    bp->ktot.assign(bp->nkinds, 0);
    auto add = [&](int kind, auto blocks) { bp_table(tab, n, blocks, bp->koff[kind], bp->ktot[kind]); };
    add(BK_FINE, [&](int i) { return (ps[i]->ni * ps[i]->nj + ET - 1) / ET; });
    add(BK_RED, [&](int i) { return ps[i]->red_blocks; });
    add(BK_ZERO, [&](int i) { return ps[i]->cs_b > 0 ? (ps[i]->ni * ps[i]->nj + ET - 1) / ET : 0; });
    for (int l = 0; l < bp->max_cs; l++) {
      auto on = [&](int i) { return l < ps[i]->cs_b; };
      add(bk_lvl(l), [&](int i) { return on(i) ? (ps[i]->lv[l].ni * ps[i]->lv[l].nj + ET - 1) / ET : 0; });
      add(bk_lvlc(l), [&](int i) { return on(i) ? (ps[i]->lv[l + 1].ni * ps[i]->lv[l + 1].nj + ET - 1) / ET : 0; });
      add(bk_half(l), [&](int i) { return on(i) ? (ps[i]->lv[l].nj * ((ps[i]->lv[l].ni + 1) / 2) + ET - 1) / ET : 0; });
    }
    SF_CUDA(cudaMalloc(&bp->d_tab, sizeof(int) * tab.size()));
    copy_wait(bp->d_tab, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, stream);
    SF_CUDA(cudaMalloc(&bp->d_koff, sizeof(int) * bp->nkinds));
    copy_wait(bp->d_koff, bp->koff.data(), sizeof(int) * bp->nkinds, cudaMemcpyHostToDevice, stream);
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return ps[x]->cd_b.total > ps[y]->cd_b.total; });
    SF_CUDA(cudaMalloc(&bp->d_order, sizeof(int) * n));
    copy_wait(bp->d_order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
    SF_CUDA(cudaMalloc(&bp->d_act_pos, sizeof(int) * (n + 1)));
    SF_CUDA(cudaMalloc(&bp->d_act_list, sizeof(int) * n));
    SF_CUDA(cudaMalloc(&bp->d_act_cnt, sizeof(int)));
    SF_CUDA(cudaMalloc(&bp->d_act_start, sizeof(int) * (size_t)bp->nkinds * (n + 1)));
    SF_CUDA(cudaMalloc(&bp->d_act_total, sizeof(int) * bp->nkinds));
    SF_CUDA(cudaMalloc(&bp->d_inst, sizeof(BPInst) * n));
    SF_CUDA(cudaMalloc(&bp->d_iters, sizeof(int) * 2 * n));
    SF_CUDA(cudaFuncSetAttribute(kb_coarse_vcycle, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)COARSE_SMEM_MAX));
    SF_CUDA(cudaMalloc(&bp->d_run, sizeof(int)));
    SF_CUDA(cudaMalloc(&bp->d_rounds, sizeof(int)));
    SF_CUDA(cudaStreamCreateWithFlags(&bp->body_stream, cudaStreamNonBlocking));
    SF_CUDA(cudaMalloc(&bp->d_prm, sizeof(BPParams)));
    SF_CUDA(cudaMalloc(&bp->d_stat, sizeof(BPStat) * n));
    SF_CUDA(cudaEventCreate(&bp->ev0));
    SF_CUDA(cudaEventCreate(&bp->ev1));
    bp_fill(bp);
    return bp;
  } catch (...) {
    batch_poisson_destroy(bp);
    throw;
  }
}

void batch_poisson_destroy(BatchPoisson* bp) {
  if (!bp) return;
  if (bp->stream) cudaStreamSynchronize(bp->stream);
  for (auto& g : bp->graphs) cudaGraphExecDestroy(g.second);
  void* ptrs[] = {bp->d_inst,      bp->d_tab,       bp->d_koff,      bp->d_order,     bp->d_iters,
                  bp->d_run,       bp->d_prm,       bp->d_stat,      bp->d_act_pos,   bp->d_act_list,
                  bp->d_act_cnt,   bp->d_act_start, bp->d_act_total, bp->d_rounds};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (bp->body_stream) cudaStreamDestroy(bp->body_stream);
  if (bp->ev0) cudaEventDestroy(bp->ev0);
  if (bp->ev1) cudaEventDestroy(bp->ev1);
  delete bp;
}

// rho of the contexts' species, the nonlinear solve of every instance and E, on the
// batch stream.  iters: PCG iterations per Newton step per instance.  Returns the time
// of the whole phase; st[i] gets each instance's Newton count, V-cycles and residuals.
float batch_poisson_step(BatchPoisson* bp, const sf_poisson_params& prm, const int* iters, sf_solve_stats* st,
                         int* status) {
  SF_REQUIRE(prm.eps > 0 && prm.tol > 0 && prm.max_it > 0, SF_ERR_ARG, "bad solver parameters");
  SF_REQUIRE(prm.linear || (prm.kTe0 > 0 && prm.n0 > 0), SF_ERR_ARG, "Boltzmann electrons need n0 > 0 and kTe0 > 0");
  cudaStream_t s = bp->stream;
  bool refill = false;
  for (int i = 0; i < bp->n; i++) refill |= charged_species(bp->ctx[i]) != bp->nspecies[i];
  if (refill) bp_fill(bp);
  BPParams h;
  h.C_n0 = QE / prm.eps * prm.n0;
  h.inv_kTe = prm.linear ? 0.0 : 1.0 / prm.kTe0;
  h.phi0 = prm.phi0;
  h.inv_eps = 1.0 / prm.eps;
  h.tol = prm.tol;
  h.max_step = prm.linear ? 1e300 : 10.0 * prm.kTe0;
  h.linear = prm.linear ? 1 : 0;
  h.max_it = prm.max_it;
  int max_iters = 1;
  std::vector<int> init(2 * bp->n);
  for (int i = 0; i < bp->n; i++) {
    SF_REQUIRE(iters[i] >= 1, SF_ERR_ARG, "PCG iterations per Newton step must be >= 1");
    max_iters = std::max(max_iters, iters[i]);
    init[i] = iters[i];
    init[bp->n + i] = bp->ctx[i]->poisson->fp64_exp ? 1 : 0;  // the contexts hold the sticky choice
  }
  cudaGraphExec_t g = bp_graph(bp, max_iters);
  SF_CUDA(cudaEventRecord(bp->ev0, s));
  SF_CUDA(cudaMemcpyAsync(bp->d_prm, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  SF_CUDA(cudaMemcpyAsync(bp->d_iters, init.data(), sizeof(int) * 2 * bp->n, cudaMemcpyHostToDevice, s));
  SF_CUDA(cudaGraphLaunch(g, s));  // the whole field phase, Newton loop included
  SF_CUDA(cudaEventRecord(bp->ev1, s));
  std::vector<BPStat> hs(bp->n);
  SF_CUDA(cudaMemcpyAsync(hs.data(), bp->d_stat, sizeof(BPStat) * bp->n, cudaMemcpyDeviceToHost, s));
  SF_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  SF_CUDA(cudaEventElapsedTime(&ms, bp->ev0, bp->ev1));
  for (int i = 0; i < bp->n; i++) {
    SfPoisson* ps = bp->ctx[i]->poisson;
    ps->rho_set = true;
    ps->prm = prm;
    ps->have_prm = true;
    ps->fp64_exp = hs[i].fp64_exp != 0;
    bp->ctx[i]->efield_set = true;
    status[i] = hs[i].status;
    st[i].newton_it = hs[i].it;
    st[i].vcycles = hs[i].vcount;
    st[i].residual = hs[i].res;
    st[i].residual_inf = hs[i].res_inf;
    st[i].initial_residual = hs[i].res0;
    st[i].ms = ms;
  }
  return ms;
}

}  // namespace sf
