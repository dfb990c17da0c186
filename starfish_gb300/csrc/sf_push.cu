// sf_push.cu -- particle push + node scatter (the KineticMaterial hot path).
//
// One call of sf_push_deposit() does, for one species, what
// KineticMaterial.updateFields() does per step (core/materials/KineticMaterial.java:117-197):
//   ParticleMover.run (:299-422)   E gather, v += q/m E dt, x += v dt, ProcessBoundary
//   updateFields(md)  (:168-197)   node scatter of the particle weights (+ u/v/w moments)
//   Material.update   (Material.java:618-632)  nd = sum(w S)/V + nd_back
//
// Kernels
//   k_push     fused push + deposit over cell-sorted SoA particles.  Particles whose
//              move neither leaves the mesh nor comes near a surface segment (checked
//              with a per-node distance map) finish here; each block accumulates its
//              tile's deposit in shared memory (32-bit halves of the fixed-point value)
//              and flushes it with one 64-bit atomic per touched node.
//   k_push_slow  the remaining particles ("slow queue"): an FP32 test first clears those
//              whose path misses every candidate segment; the rest run in FP64 with the
//              reference's exact surface-hit and domain-exit logic, up to 10 bounces.
//   k_finalize  int64 fixed-point counts -> FP64 density (and mean velocities).
// The deposit is an integer sum, so node densities are bit-identical run to run.
#include <climits>
#include <mutex>
#include <string>
#include <cmath>

#include "sf_internal.h"

using namespace sf;

namespace {

constexpr int PB = 256;            // threads per block
constexpr int PPT = 4;             // particles per thread per tile
constexpr int TILE = PB * PPT;     // particles per block tile
constexpr int SBOX = 4096;         // shared-memory deposit box (nodes)
constexpr int SLOW_THREADS = 128;  // threads per block of the exact-path kernels


// Deposit quantisation of every path: S in [0,1] -> round(S * 2^22), at most 2^22 - 1, so
// that the 32-bit shared-memory sum over the TILE = 1024 particles of a tile cannot wrap;
// the values are scaled by 2^9 into the 2^31 fixed point of the global counts (DEP_SCALE).
constexpr int TILE_SHIFT = 9;
__device__ __forceinline__ unsigned quant22(float w) {
  return min(__float2uint_rn(w * 4194304.0f), 4194303u);
}

// Bilinear weights of the scatter (Field2D.scatter, core/domain/Field2D.java:244-295):
// XY plain; RZ/ZR with Ruyten's eq. 4.2 in the radial direction, written relative to
// the cell's lower radius rm so that FP32 keeps its precision away from the axis:
//   d = 1 - (1-f)(4 rm + (2-f) dr) / (2 (2 rm + dr))
template <int DOM>
__device__ __forceinline__ void scatter_weights(float fx, float fy, int i, int j, const PushArgs& a,
                                                float& di, float& dj) {
  di = fx;
  dj = fy;
  if (DOM == SF_DOMAIN_RZ) {
    float rm = a.r0x + (float)i * a.dx;
    di = 1.f - 0.5f * (1.f - fx) * (4.f * rm + (2.f - fx) * a.dx) / (2.f * rm + a.dx);
  } else if (DOM == SF_DOMAIN_ZR) {
    float rm = a.r0y + (float)j * a.dy;
    dj = 1.f - 0.5f * (1.f - fy) * (4.f * rm + (2.f - fy) * a.dy) / (2.f * rm + a.dy);
  }
}

__device__ __forceinline__ float2 gather_E(const MeshView& m, int i, int j, float fx, float fy) {
  // Field2D.gather (Field2D.java:318-350); at lc = n-1 the cell is n-2 with fraction 1,
  // which gives gather_safe's value (:371-390).
  return gather_efield(m.E, m.ni, i, j, fx, fy);
}

struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// ---------------------------------------------------------------------------------
// fused push + deposit
// ---------------------------------------------------------------------------------
// Deposit accumulation: each particle adds round(S * 2^22) (quant22) to its four corner
// nodes.  Inside a block the tile's box of nodes is accumulated in shared memory with one
// 32-bit atomic per corner (1024 particles of at most 2^22 - 1 cannot overflow), then
// flushed with one 64-bit global atomic per touched node, scaled by 2^9 into the global
// 2^31 fixed point.  Tiles whose box does not fit (unsorted input) add the same scaled
// values with 64-bit global atomics per corner, so both routes give the same integers.
__device__ bool may_hit_fp32(const MeshView& m, int i, int j, float fx, float fy, float gx, float gy);

// One tile (TILE particles from t0) of the fused push + deposit: load, push, fast-path
// test, enqueue of slow candidates, shared-memory deposit of the tile's box and its
// flush.  Shared by k_push (one mesh) and k_push_batch (many instances).  PRE: a
// particle that fails the distance test is given the exact path's FP32 pre-filter here,
// and finishes here when no candidate segment can be on its path (moves of many cells,
// as in small meshes at large dt, would otherwise mostly queue for the exact path).
// W: per-particle weights (P.w): each deposit, moment and total is scaled by the particle's
// fraction of the species weight, and st_w sums the fractions (st_n counts particles).
template <int DOM, bool STATS, bool MOM, bool PRE = false, bool W = false>
__device__ __forceinline__ void push_tile(const MeshView& m, const ParticlesView& P, const PushArgs& a, int64_t t0,
                                          unsigned long long* __restrict__ count, long long* __restrict__ mom,
                                          int* __restrict__ slow_idx, unsigned long long* __restrict__ counters,
                                          const SampleView& smp, unsigned* acc,
                                          int (*sred)[PB / 32], Kahan& st_px, Kahan& st_py, Kahan& st_pz, Kahan& st_e,
                                          unsigned& st_n, Kahan& st_w) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;
  const size_t nn = (size_t)m.ni * m.nj;
  int pi[PPT], pj[PPT];
  float pfx[PPT], pfy[PPT];
  float pv[PPT][3];
  bool dep[PPT];
  int imin = INT_MAX, imax = -1, jmin = INT_MAX, jmax = -1;
  // load phase: all of the thread's particles are requested before any is used, so
  // each warp keeps PPT independent streams of loads in flight (streaming hints keep
  // L2 for the field and the deposit grid)
  uint32_t lcell[PPT];
  float2 lfrac[PPT], lvxy[PPT];
  float lvz[PPT];
  float pw[PPT];  // weight fractions (W)
  // the tile's arrays from its first particle: 32-bit indices inside the tile
  uint32_t* __restrict__ tcell = P.cell + t0;
  float2* __restrict__ tfrac = P.frac + t0;
  float2* __restrict__ tvxy = P.vxy + t0;
  float* __restrict__ tvz = P.vz + t0;
  const int nrem = (int)min(P.n - t0, (int64_t)TILE);
#pragma unroll
  for (int k = 0; k < PPT; k++) {
    const int q = k * PB + (int)threadIdx.x;
    lcell[k] = DEAD;
    lvz[k] = 0.f;
    pw[k] = 1.f;
    if (q < nrem) {
      lcell[k] = __ldcs(tcell + q);
      lfrac[k] = __ldcs(tfrac + q);
      lvxy[k] = __ldcs(tvxy + q);
      if (DOM != SF_DOMAIN_XY || STATS || MOM) lvz[k] = __ldcs(tvz + q);
      if (W) pw[k] = P.w ? __ldcs(P.w + t0 + q) : 1.f;  // (a batch mixes weighted and uniform species)
    }
  }
#pragma unroll
  for (int k = 0; k < PPT; k++) {
    const int q = k * PB + (int)threadIdx.x;
    dep[k] = false;
    pi[k] = pj[k] = 0;
    pfx[k] = pfy[k] = 0.f;
    int status = 0;  // 1 finished here, 2 exact path, 3 removed at a domain face
    if (q < nrem) {
      const uint32_t c = lcell[k];
      if (c != DEAD) {
        const int i = cell_i(c), j = cell_j(c);
        const float2 f = lfrac[k];
        float2 v = lvxy[k];
        // velocity update (KineticMaterial.java:336-346); B = 0
        const float2 e = gather_E(m, i, j, f.x, f.y);
        v.x += a.qm_dt * e.x;
        v.y += a.qm_dt * e.y;
        float vz = lvz[k];
        // move in logical coordinates (x += v dt; XtoL)
        float nfx, nfy, nvx = v.x, nvy = v.y, nvz = vz;
        float gx, gy;  // the new position in cells from (i, j), before reduction
        if (DOM == SF_DOMAIN_XY) {
          nfx = f.x + v.x * a.dt_dx;
          nfy = f.y + v.y * a.dt_dy;
          gx = nfx;
          gy = nfy;
        } else if (DOM == SF_DOMAIN_ZR) {
          // rotateToZR (KineticMaterial.java:444-462) relative to the cell radius rj
          nfx = f.x + v.x * a.dt_dx;
          // one reciprocal square root and one approximate division (2 ulp) instead of a
          // square root and four IEEE divisions
          const float rj = a.r0y + (float)j * a.dy;
          const float A = vz * a.dt;
          const float dl = f.y * a.dy + v.y * a.dt;
          const float B = rj + dl;
          const float s2 = A * A + B * B;
          const float ir = s2 > 0.f ? rsqrtf(s2) : 0.f;
          const float R = s2 * ir;
          const float den = R + rj;
          const float rrel = den > 0.f ? __fdividef(A * A + dl * (2.f * rj + dl), den) : 0.f;
          nfy = rrel * m.inv_dy;
          const float cs = R > 0.f ? B * ir : 1.f, sn = R > 0.f ? A * ir : 0.f;
          nvy = cs * v.y + sn * vz;
          nvz = -sn * v.y + cs * vz;
          gx = nfx;
          gy = nfy;
        } else {
          // rotateToRZ (KineticMaterial.java:424-442), radius along x
          nfy = f.y + v.y * a.dt_dy;
          const float ri = a.r0x + (float)i * a.dx;
          const float A = vz * a.dt;
          const float dl = f.x * a.dx + v.x * a.dt;
          const float B = ri + dl;
          const float s2 = A * A + B * B;
          const float ir = s2 > 0.f ? rsqrtf(s2) : 0.f;
          const float R = s2 * ir;
          const float den = R + ri;
          const float rrel = den > 0.f ? __fdividef(A * A + dl * (2.f * ri + dl), den) : 0.f;
          nfx = rrel * m.inv_dx;
          const float cs = R > 0.f ? B * ir : 1.f, sn = R > 0.f ? A * ir : 0.f;
          nvx = cs * v.x + sn * vz;
          nvz = -sn * v.x + cs * vz;
          gx = nfx;
          gy = nfy;
        }
        float fdi = floorf(nfx), fdj = floorf(nfy);
        nfx -= fdi;
        nfy -= fdj;
        if (nfx >= 1.f) { nfx -= 1.f; fdi += 1.f; }
        if (nfy >= 1.f) { nfy -= 1.f; fdj += 1.f; }
        const int di = (int)fdi, dj = (int)fdj;
        const int i2 = i + di, j2 = j + dj;
        const int span = max(abs(di), abs(dj)) + 1;
        const bool inside = (i2 >= 0) & (j2 >= 0) & (i2 <= m.ni - 2) & (j2 <= m.nj - 2);
        // the tile's least distance first (L1-resident); the node's own only near segments
        bool clear = (int)__ldg(&m.seg_dist_tile[(j >> 4) * ((m.ni + 15) >> 4) + (i >> 4)]) > span ||
                     (int)__ldg(&m.seg_dist[j * m.ni + i]) > span;
        if (PRE && !clear) clear = !may_hit_fp32(m, i, j, f.x, f.y, gx, gy);
        if (inside && clear) {
          __stcs(tcell + q, pack_cell(i2, j2));
          __stcs(tfrac + q, make_float2(nfx, nfy));
          __stcs(tvxy + q, make_float2(nvx, nvy));
          if (DOM != SF_DOMAIN_XY) __stcs(tvz + q, nvz);
          status = 1;
          dep[k] = true;
          pi[k] = i2;
          pj[k] = j2;
          pfx[k] = nfx;
          pfy[k] = nfy;
          pv[k][0] = nvx;
          pv[k][1] = nvy;
          pv[k][2] = nvz;
          imin = min(imin, i2);
          imax = max(imax, i2);
          jmin = min(jmin, j2);
          jmax = max(jmax, j2);
          if (STATS) {
            st_n++;
            const float wk = pw[k];
            if (W) st_w.add(wk);
            st_px.add(W ? wk * nvx : nvx);
            st_py.add(W ? wk * nvy : nvy);
            st_pz.add(W ? wk * nvz : nvz);
            st_e.add((W ? wk : 1.f) * sqrtf(nvx * nvx + nvy * nvy + nvz * nvz));
          }
        } else if (!inside && clear && m.all_delete) {
          // no candidate segment on the way and every domain face removes particles
          // (KineticMaterial.java:614-746: OPEN/DIRICHLET/... return false)
          tcell[q] = DEAD;
          status = 3;
        } else {
          // exact path later: keep the old position, store the updated velocity
          tvxy[q] = v;
          status = 2;
        }
      }
    }
    const unsigned ms = __ballot_sync(FULL, status == 2);
    if (ms) {
      const int leader = __ffs(ms) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&counters[0], (unsigned long long)__popc(ms));
      base = __shfl_sync(FULL, base, leader);
      if (status == 2) slow_idx[base + __popc(ms & ((1u << lane) - 1u))] = (int)t0 + q;
    }
    const unsigned md = __ballot_sync(FULL, status == 3);
    if (md && lane == __ffs(md) - 1) atomicAdd(&counters[1], (unsigned long long)__popc(md));
  }
  // ---- block bounding box of this tile's deposits ----
  imin = __reduce_min_sync(FULL, imin);
  jmin = __reduce_min_sync(FULL, jmin);
  imax = __reduce_max_sync(FULL, imax);
  jmax = __reduce_max_sync(FULL, jmax);
  if (lane == 0) {
    sred[0][wid] = imin;
    sred[1][wid] = jmin;
    sred[2][wid] = imax;
    sred[3][wid] = jmax;
  }
  __syncthreads();
  imin = sred[0][0];
  jmin = sred[1][0];
  imax = sred[2][0];
  jmax = sred[3][0];
#pragma unroll
  for (int w = 1; w < PB / 32; w++) {
    imin = min(imin, sred[0][w]);
    jmin = min(jmin, sred[1][w]);
    imax = max(imax, sred[2][w]);
    jmax = max(jmax, sred[3][w]);
  }
  const int bw = imax - imin + 2, bh = jmax - jmin + 2;
  const bool any = imax >= 0;
  const bool use_smem = any && (bw * bh <= SBOX);
  // acc[] is all zero here: zeroed once by the kernel, and the flush below clears every
  // node of the box it reads
  if (any) {
#pragma unroll
    for (int k = 0; k < PPT; k++) {
      // scatter skip rule at the far mesh edges (lc >= n-1 is not scattered)
      // macroparticles per cell at (int) lc (KineticMaterial.updateSamples)
      if (MOM && dep[k] && smp.mpc)
        atomicAdd(&smp.mpc[(pj[k] + (pfy[k] >= 1.f)) * m.ni + pi[k] + (pfx[k] >= 1.f)], 1u);
      const bool d = dep[k] && !((pfx[k] >= 1.f && pi[k] == m.ni - 2) || (pfy[k] >= 1.f && pj[k] == m.nj - 2));
      if (!d) continue;
      float wx, wy;
      scatter_weights<DOM>(pfx[k], pfy[k], pi[k], pj[k], a, wx, wy);
      const float wk = pw[k];
      const unsigned q[4] = {quant22((W ? wk : 1.f) * ((1.f - wx) * (1.f - wy))),
                             quant22((W ? wk : 1.f) * (wx * (1.f - wy))), quant22((W ? wk : 1.f) * (wx * wy)),
                             quant22((W ? wk : 1.f) * ((1.f - wx) * wy))};
      if (MOM) {
        const float s[4] = {(W ? wk : 1.f) * ((1.f - wx) * (1.f - wy)), (W ? wk : 1.f) * (wx * (1.f - wy)),
                            (W ? wk : 1.f) * (wx * wy), (W ? wk : 1.f) * ((1.f - wx) * wy)};
        const int base = pj[k] * m.ni + pi[k];
        const int off[4] = {0, 1, m.ni + 1, m.ni};
#pragma unroll
        for (int cc = 0; cc < 4; cc++)
#pragma unroll
          for (int dd = 0; dd < 3; dd++)
            atomicAdd((unsigned long long*)&mom[dd * nn + base + off[cc]],
                      (unsigned long long)__float2ll_rn(s[cc] * pv[k][dd] * 65536.0f));
        if (smp.mom2)
#pragma unroll
          for (int cc = 0; cc < 4; cc++)
#pragma unroll
            for (int dd = 0; dd < 3; dd++)
              atomicAdd(&smp.mom2[dd * nn + base + off[cc]],
                        __float2ull_rn(s[cc] * pv[k][dd] * pv[k][dd] * (float)MOM2_SCALE));
      }
      if (use_smem) {
        const int l = (pj[k] - jmin) * bw + (pi[k] - imin);
        const int off[4] = {0, 1, bw + 1, bw};
#pragma unroll
        for (int cc = 0; cc < 4; cc++) {
          atomicAdd(&acc[l + off[cc]], q[cc]);
        }
      } else {
        const size_t u = (size_t)pj[k] * m.ni + pi[k];
        const size_t off[4] = {0, 1, (size_t)m.ni + 1, (size_t)m.ni};
#pragma unroll
        for (int cc = 0; cc < 4; cc++) atomicAdd(&count[u + off[cc]], (unsigned long long)q[cc] << TILE_SHIFT);
      }
    }
  }
  __syncthreads();
  if (use_smem) {
    // row = q / bw by a multiply-high with mg = ceil(2^32 / bw), exact while q * bw < 2^32
    // (q < SBOX = 4096 and bw <= SBOX)
    const uint32_t mg = 0xffffffffu / (uint32_t)bw + 1u;
    for (int q = threadIdx.x; q < bw * bh; q += PB) {
      const unsigned a32 = acc[q];
      if (a32) {
        acc[q] = 0u;
        const int r = (int)__umulhi((uint32_t)q, mg);
        atomicAdd(&count[(size_t)(jmin + r) * m.ni + imin + (q - r * bw)], (unsigned long long)a32 << TILE_SHIFT);
      }
    }
  }
  __syncthreads();
}

// L2 prefetch of a tile's particle arrays (one bulk prefetch per array, issued by one
// thread) while the block pushes its current tile.  Only whole 16-byte groups of the
// tile's particles are requested, all inside [0, P.n).
template <int DOM, bool STATS, bool MOM, bool W>
__device__ __forceinline__ void prefetch_tile(const ParticlesView& P, int64_t t0) {
  if (t0 >= P.n) return;
  const uint32_t nrem = (uint32_t)min(P.n - t0, (int64_t)TILE);
  prefetch_l2(P.cell + t0, (nrem * 4u) & ~15u);
  prefetch_l2(P.frac + t0, (nrem * 8u) & ~15u);
  prefetch_l2(P.vxy + t0, (nrem * 8u) & ~15u);
  if (DOM != SF_DOMAIN_XY || STATS || MOM) prefetch_l2(P.vz + t0, (nrem * 4u) & ~15u);
  if (W && P.w) prefetch_l2(P.w + t0, (nrem * 4u) & ~15u);
}

template <int DOM, bool STATS, bool MOM, bool W>
__global__ void __launch_bounds__(PB, 4) k_push(MeshView m, ParticlesView P, PushArgs a,
                                              unsigned long long* __restrict__ count,
                                              long long* __restrict__ mom, int* __restrict__ slow_idx,
                                              unsigned long long* __restrict__ counters,
                                              double* __restrict__ stats_partial, SampleView smp) {
  __shared__ unsigned acc[SBOX];
  __shared__ int sred[4][PB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;
  Kahan st_px, st_py, st_pz, st_e, st_w;
  unsigned st_n = 0;
  for (int q = threadIdx.x; q < SBOX; q += PB) acc[q] = 0u;
  __syncthreads();

  const int64_t stride = (int64_t)gridDim.x * TILE;
  for (int64_t t0 = (int64_t)blockIdx.x * TILE; t0 < P.n; t0 += stride) {
    if (threadIdx.x == 0) prefetch_tile<DOM, STATS, MOM, W>(P, t0 + stride);
    // the in-tile pre-filter pays on RZ/ZR meshes whose walls run along dense gas (the jet's
    // inlet plane: push 0.198 -> 0.228 ms, exact path 0.21 -> 0.09 ms per step); on the XY
    // workload it made the push slower (0.598 -> 0.647 ms) than the queue it saves
    push_tile<DOM, STATS, MOM, DOM != SF_DOMAIN_XY, W>(m, P, a, t0, count, mom, slow_idx, counters, smp, acc, sred, st_px, st_py,
                                         st_pz, st_e, st_n, st_w);
  }
  if (STATS) {
    // block reduction of the per-thread sums (FP64 from here on); the first is the particle
    // count, or with weights the sum of the weight fractions
    double vals[5] = {W ? (double)st_w.s - st_w.c : (double)st_n, (double)st_px.s - st_px.c, (double)st_py.s - st_py.c,
                      (double)st_pz.s - st_pz.c, (double)st_e.s - st_e.c};
    __shared__ double sd[5][PB / 32];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      double x = vals[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULL, x, o);
      if (lane == 0) sd[q][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
      double x = 0;
      for (int w = 0; w < PB / 32; w++) x += sd[threadIdx.x][w];
      stats_partial[(size_t)blockIdx.x * 8 + threadIdx.x] = x;
    }
  }
}

// ---------------------------------------------------------------------------------
// exact path (FP64): ProcessBoundary with surface segments and domain faces
// ---------------------------------------------------------------------------------
struct Seg64 {
  double x1[2], x2[2];
};

__device__ inline void seg_normal_tangent(const Seg4 s, double n[3], double tg[3]) {
  // LinearSegment constructor (LinearSegment.java:22-46)
  double dx = s.z - s.x, dy = s.w - s.y;
  double len = sqrt(dx * dx + dy * dy);
  dx /= len;
  dy /= len;
  tg[0] = dx; tg[1] = dy; tg[2] = 0;
  n[0] = -dy; n[1] = dx; n[2] = 0;
}

// Utils.SampleMaxwSpeed (core/common/Utils.java:69-87), rejection bounded at 10^4 tries.
// A sampled speed needs no more than FP32: the draws and the acceptance test are FP32
// (f/f_max = (v/v_th)^2 e^(1 - (v/v_th)^2), the reference's ratio in closed form).
__device__ float sample_maxw_speed(Philox& r, float v_th) {
  float x = 1.f;  // v / v_th
  for (int tries = 0; tries < 10000; tries++) {
    x = r.uniformf() * 6.f;
    if (x * x * __expf(1.f - x * x) > r.uniformf()) break;
  }
  return x * v_th;
}


// Conservative FP32 test of one segment (a, b) against the straight path f -> g, all in
// cells relative to the particle's node: 0 means the two cannot intersect by the rule of
// LinearSegment.intersect (both parameters within [-1e-7, 1 + 1e-7], Segment.java and
// KineticMaterial.java:480-515); 1 means they intersect with both parameters inside (0, 1)
// by more than the error bound, so the exact path takes this crossing with *tseg, *tpart
// (the segment and path parameters) within *marg of its values; 2 is undecided.
// The bound is a forward error bound of the FP32 cross products.  With u = 2^-24,
// A = 1 + the largest endpoint coordinate and G = 1 + the largest path coordinate: the
// endpoints carry u A (one rounding of integer cell + fraction), the path end 9 u G (the
// FP32 move against the FP64 one), so the denominator r x s is off by at most 64 u G A, the
// path numerator q x s by 24 u A^2 and the segment numerator q x r by 26 u A G (each
// including the products' own roundings).  Near-parallel paths are undecided.
__device__ __forceinline__ int seg_class_fp32(float ax, float ay, float bx, float by, float fx, float fy, float gx,
                                              float gy, float* tseg, float* tpart = nullptr, float* marg = nullptr) {
  const float rx = gx - fx, ry = gy - fy;
  const float sx = bx - ax, sy = by - ay;
  const float den = rx * sy - ry * sx;
  const float qx = ax - fx, qy = ay - fy;
  const float tn = qx * sy - qy * sx;  // t_part * den
  const float un = qx * ry - qy * rx;  // t_seg * den
  const float lim = fabsf(den);
  const float U = 5.9604645e-8f;  // 2^-24
  const float A1 = fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fmaxf(fabsf(bx), fabsf(by))) + 1.f;
  const float G1 = fmaxf(fmaxf(fabsf(gx), fabsf(gy)), fmaxf(fabsf(fx), fabsf(fy))) + 1.f;
  const float d_den = 64.f * U * G1 * A1;
  const float rs = (fabsf(rx) + fabsf(ry)) * (fabsf(sx) + fabsf(sy));
  if (lim <= 2.f * d_den || lim <= 1e-5f * rs) return 2;  // (near) parallel
  // the reference's acceptance window (1e-7 of each parameter range), with room for its own
  // FP64 rounding
  const float win = 1.02e-7f * lim;
  const float tol_p = win + 24.f * U * A1 * A1 + d_den;
  const float tol_s = win + 26.f * U * A1 * G1 + d_den;
  const float sgn = den > 0.f ? 1.f : -1.f;
  const float t1 = tn * sgn, t0 = un * sgn;
  if (!(t1 >= -tol_p && t1 <= lim + tol_p && t0 >= -tol_s && t0 <= lim + tol_s)) return 0;
  if (t1 >= tol_p && t1 <= lim - tol_p && t0 >= tol_s && t0 <= lim - tol_s) {
    *tseg = t0 / lim;
    if (tpart) *tpart = t1 / lim;
    if (marg) *marg = fmaxf(tol_p, tol_s) / lim;
    return 1;
  }
  return 2;
}

__device__ __forceinline__ bool seg_may_cross_fp32(float ax, float ay, float bx, float by, float fx, float fy,
                                                   float gx, float gy) {
  float t;
  return seg_class_fp32(ax, ay, bx, by, fx, fy, gx, gy, &t) != 0;
}

// Visits the DIRICHLET/SINK segments that KineticMaterial.ProcessBoundary collects for
// the node box [i_min..i_max] x [j_min..j_max] (KineticMaterial.java:480-515); f(s)
// returning true stops the walk.  With few segments all of them are visited directly:
// a segment met by a path inside the box passes within 1.01 cells of a box node, so
// Mesh.setNodeControlVolumes lists it there and the set of possible hits is the same.
// With many segments the node lists are walked, testing each segment once (a short
// list of visited ids; repeats beyond it are harmless re-tests).
constexpr int SMALL_NSEG = 64;
template <typename F>
__device__ inline void for_each_candidate(const MeshView& m, int i_min, int i_max, int j_min, int j_max, F&& f) {
  if (m.nseg <= SMALL_NSEG) {
    for (int s = 0; s < m.nseg; s++) {
      const int bt = m.seg_btype[s];
      if (bt != SF_BT_DIRICHLET && bt != SF_BT_SINK) continue;
      if (f(s)) return;
    }
    return;
  }
  constexpr int SEEN = 16;
  int seen[SEEN];
  int nseen = 0;
  for (int i = i_min; i <= i_max; i++)
    for (int j = j_min; j <= j_max; j++) {
      const int u = j * m.ni + i;
      for (int k = m.node_seg_ptr[u]; k < m.node_seg_ptr[u + 1]; k++) {
        const int s = m.node_seg_idx[k];
        const int bt = m.seg_btype[s];
        if (bt != SF_BT_DIRICHLET && bt != SF_BT_SINK) continue;
        bool dup = false;
        for (int q = 0; q < nseen; q++) dup |= (seen[q] == s);
        if (dup) continue;
        if (nseen < SEEN) seen[nseen++] = s;
        if (f(s)) return;
      }
    }
}

// returns alive; follows KineticMaterial.ProcessBoundary (KineticMaterial.java:471-750)
__device__ bool process_boundary(const MeshView& m, const SlowArgs& sa, const PushArgs& a, double pos[2],
                                 double vel[3], double lc[2], double& pdt, const double old[2],
                                 const double lc_old[2], Philox& rng, bool& periodic) {
  const double dt0 = pdt;
  pdt = 0;
  int i_min = (int)fmin(lc[0], lc_old[0]), i_max = (int)fmax(lc[0], lc_old[0]);
  int j_min = (int)fmin(lc[1], lc_old[1]), j_max = (int)fmax(lc[1], lc_old[1]);
  if (i_min < 0) i_min = 0;
  if (j_min < 0) j_min = 0;
  if (i_max >= m.ni) i_max = m.ni - 1;
  if (j_max >= m.nj) j_max = m.nj - 1;
  double tp_min = 2.0, tsurf_min = 0;
  int seg_min = -1;
  // the path in cells from the old position's cell: segments that the FP32 test clears
  // cannot intersect it, and their FP64 intersection (which would give no hit) is skipped
  const double bi = floor(lc_old[0]), bj = floor(lc_old[1]);
  const int io = (int)bi, jo = (int)bj;
  const float ofx = (float)(lc_old[0] - bi), ofy = (float)(lc_old[1] - bj);
  const float ngx = (float)(lc[0] - bi), ngy = (float)(lc[1] - bj);
  for_each_candidate(m, i_min, i_max, j_min, j_max, [&](int s) {
    const SegLC sl = m.seg_lc[s];
    if (!seg_may_cross_fp32((float)(sl.i1 - io) + sl.f1, (float)(sl.j1 - jo) + sl.g1, (float)(sl.i2 - io) + sl.f2,
                            (float)(sl.j2 - jo) + sl.g2, ofx, ofy, ngx, ngy))
      return false;
    const Seg4 sxy = m.seg_xy[s];
    double t[2];
    seg_intersect(sxy, old, pos, t);
    const double t_part = t[1];
    if (t_part > 0) {
      if (t_part < FLT_EPS_REF) {  // leaving the surface it starts on (acs > 0): no hit
        double n[3], tg[3];
        seg_normal_tangent(sxy, n, tg);
        const double acs = (n[0] * vel[0] + n[1] * vel[1]) / sqrt(vel[0] * vel[0] + vel[1] * vel[1]);
        if (acs > 0) return false;
      }
      if (t_part < tp_min) {
        tp_min = t_part;
        tsurf_min = t[0];
        seg_min = s;
      }
    }
    return false;
  });
  bool alive = true;
  if (seg_min >= 0) {
    tp_min *= 0.9999;
    pos[0] = old[0] + tp_min * (pos[0] - old[0]);
    pos[1] = old[1] + tp_min * (pos[1] - old[1]);
    lc[0] = (pos[0] - m.x0[0]) * m.inv_dh[0];
    lc[1] = (pos[1] - m.x0[1]) * m.inv_dh[1];
    pdt = dt0 * (1 - tp_min);
    if (lc[0] < 0 && lc[0] > -FLT_EPS_REF) lc[0] = 0;
    if (lc[1] < 0 && lc[1] > -FLT_EPS_REF) lc[1] = 0;
    const int model = sa.sv.model[seg_min];
    const Seg4 sxy = m.seg_xy[seg_min];
    double n[3], tg[3];
    seg_normal_tangent(sxy, n, tg);
    const double v_in = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    switch (model) {
      case SF_SURF_PASS:
      case SF_SURF_NONE: alive = true; break;
      case SF_SURF_SPECULAR: {  // SurfaceInteraction.java:104-150
        const double mag = sqrt(vel[0] * vel[0] + vel[1] * vel[1]) * 1.4142135623730951;
        vel[0] += n[0] * mag;
        vel[1] += n[1] * mag;
        alive = true;
        break;
      }
      case SF_SURF_DIFFUSE: {  // SurfaceInteraction.java:153-213 (cosine emission)
        const float4 pr = sa.sv.param[seg_min];
        const double v_refl = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]) * pr.y;
        const double v_diff = (double)sample_maxw_speed(rng, pr.x);
        const double v_mag = v_refl + pr.z * (v_diff - v_refl);
        // Vec.lambertianVector (core/common/Vec.java:450-471), the random direction in FP32
        float cosphi = sqrtf(1.f - rng.uniformf());
        if (cosphi > 0.99999f) cosphi = 0.99999f;
        const float theta = 2.f * (float)PI * rng.uniformf();
        const float sinphi = sqrtf(1.f - cosphi * cosphi);
        float st, ct;
        __sincosf(theta, &st, &ct);
        const double c_t = (double)(ct * sinphi), c_n = (double)cosphi, c_p = (double)(st * sinphi);
        const double pz[3] = {0, 0, 1};
        for (int q = 0; q < 3; q++) vel[q] = v_mag * (c_t * tg[q] + c_n * n[q] + c_p * pz[q]);
        alive = true;
        break;
      }
      default: alive = false; break;  // ABSORB
    }
    if (sa.sv.product && (model == SF_SURF_SPECULAR || model == SF_SURF_DIFFUSE)) {
      const int2 pe = sa.sv.product[seg_min];
      if (pe.x >= 0) {
        // species change (SurfaceInteraction.java:128-142, 175-193): the particle leaves
        // and (int)(spwt / spwt_product + rnd) product particles start from the hit point
        // (the ParticleListSource of the product, emitted with Source.sampleKinetic's
        // 1e-6 dt push off and addParticle's rewind): specular ones with the reflected
        // velocity, diffuse ones each with its own cosine-law direction and speed
        const ProductView& Q = sa.sv.prod[pe.x];
        const float vthp = __int_as_float(pe.y);
        const float4 pr = sa.sv.param[seg_min];
        const int count = (int)(a.spwt / Q.spwt + rng.uniform());
        const double hx = sxy.x + tsurf_min * (sxy.z - sxy.x), hy = sxy.y + tsurf_min * (sxy.w - sxy.y);
        for (int k = 0; k < count; k++) {
          double v[3] = {vel[0], vel[1], vel[2]};
          if (model == SF_SURF_DIFFUSE) {
            const double v_refl = v_in * pr.y;
            const double v_mag = v_refl + pr.z * ((double)sample_maxw_speed(rng, vthp) - v_refl);
            float cosphi = sqrtf(1.f - rng.uniformf());
            if (cosphi > 0.99999f) cosphi = 0.99999f;
            const float theta = 2.f * (float)PI * rng.uniformf();
            const float sinphi = sqrtf(1.f - cosphi * cosphi);
            float st, ct;
            __sincosf(theta, &st, &ct);
            const double c_t = (double)(ct * sinphi), c_n = (double)cosphi, c_p = (double)(st * sinphi);
            const double pz[3] = {0, 0, 1};
            for (int q = 0; q < 3; q++) v[q] = v_mag * (c_t * tg[q] + c_n * n[q] + c_p * pz[q]);
          }
          const double px = hx + v[0] * 1e-6 * a.dt64, py = hy + v[1] * 1e-6 * a.dt64;
          const int64_t d = Q.P.n + (int64_t)atomicAdd(Q.added, 1ULL);
          if (d >= Q.cap) continue;  // counted: the host reports the overflow
          const double lx = fmin(fmax((px - m.x0[0]) * m.inv_dh[0], 0.0), m.ni - 1.0);
          const double ly = fmin(fmax((py - m.x0[1]) * m.inv_dh[1], 0.0), m.nj - 1.0);
          const int ci = min((int)lx, m.ni - 2), cj = min((int)ly, m.nj - 2);
          const float fx = (float)(lx - ci), fy = (float)(ly - cj);
          const float2 e = gather_E(m, ci, cj, fx, fy);
          Q.P.cell[d] = pack_cell(ci, cj);
          Q.P.frac[d] = make_float2(fx, fy);
          Q.P.vxy[d] = make_float2((float)v[0] - Q.qm_halfdt * e.x, (float)v[1] - Q.qm_halfdt * e.y);
          Q.P.vz[d] = (float)v[2];
          if (Q.P.w) Q.P.w[d] = 1.f;  // products at their species weight
        }
        alive = false;
      }
    }
    if (!alive) atomicAdd(&sa.stats_slow[5], a.spwt * a.charge);
    if (m.seg_btype[seg_min] == SF_BT_SINK) alive = false;
    atomicAdd(&sa.sv.flux[2 * seg_min], a.spwt * (1 - tsurf_min));
    atomicAdd(&sa.sv.flux[2 * seg_min + 1], a.spwt * tsurf_min);
    if (!alive) {
      atomicAdd(&sa.sv.deposit[2 * seg_min], a.spwt * (1 - tsurf_min));
      atomicAdd(&sa.sv.deposit[2 * seg_min + 1], a.spwt * tsurf_min);
      return false;
    }
  }
  if (lc[0] < 0 || lc[1] < 0 || lc[0] >= m.ni - 1 || lc[1] >= m.nj - 1) {
    double t_right = 99, t_top = 99, t_left = 99, t_bottom = 99;
    if (lc[0] >= m.ni - 1) t_right = (m.ni - 1.0 - lc_old[0]) / (lc[0] - lc_old[0]);
    if (lc[1] >= m.nj - 1) t_top = (m.nj - 1.0 - lc_old[1]) / (lc[1] - lc_old[1]);
    if (lc[0] < 0) t_left = lc_old[0] / (lc_old[0] - lc[0]);
    if (lc[1] < 0) t_bottom = lc_old[1] / (lc_old[1] - lc[1]);
    int face = SF_FACE_RIGHT;
    double t = t_right;
    if (t_top < t) { face = SF_FACE_TOP; t = t_top; }
    if (t_left < t) { face = SF_FACE_LEFT; t = t_left; }
    if (t_bottom < t) { face = SF_FACE_BOTTOM; t = t_bottom; }
    lc[0] = lc_old[0] + t * (lc[0] - lc_old[0]);
    lc[1] = lc_old[1] + t * (lc[1] - lc_old[1]);
    if (lc[0] < 0) lc[0] = 0;
    else if (lc[0] > m.ni - 1) lc[0] = m.ni - 1;
    if (lc[1] < 0) lc[1] = 0;
    else if (lc[1] > m.nj - 1) lc[1] = m.nj - 1;
    pos[0] = m.x0[0] + lc[0] * m.dh[0];
    pos[1] = m.x0[1] + lc[1] * m.dh[1];
    pdt = dt0 * (1 - t);
    int i = (int)lc[0], j = (int)lc[1];
    if (face == SF_FACE_TOP) j++;
    if (face == SF_FACE_RIGHT) i++;
    if (i < 0) i = 0;
    if (j < 0) j = 0;
    if (i >= m.ni - 1) i = m.ni - 1;
    if (j >= m.nj - 1) j = m.nj - 1;
    const int idx = (face == SF_FACE_LEFT || face == SF_FACE_RIGHT) ? j : i;
    const int type = m.face_type[face * m.nmax + idx];
    switch (type) {
      case SF_DB_SYMMETRY: {  // Vec.mirror about UniformMesh.faceNormal
        double n[3] = {0, 0, 0};
        if (face == SF_FACE_LEFT) n[0] = 1;
        else if (face == SF_FACE_RIGHT) n[0] = -1;
        else if (face == SF_FACE_BOTTOM) n[1] = 1;
        else n[1] = -1;
        const double tm = vel[0] * n[0] + vel[1] * n[1] + vel[2] * n[2];
        for (int q = 0; q < 3; q++) {
          const double tq = n[q] * tm;
          vel[q] = -tq + (vel[q] - tq);
        }
        return true;
      }
      case SF_DB_PERIODIC: {
        const double Lx = (m.ni - 1) * m.dh[0], Ly = (m.nj - 1) * m.dh[1];
        if (face == SF_FACE_LEFT) pos[0] += Lx;
        else if (face == SF_FACE_RIGHT) pos[0] -= Lx;
        else if (face == SF_FACE_BOTTOM) pos[1] += Ly;
        else pos[1] -= Ly;
        periodic = true;
        return true;
      }
      default: return false;  // OPEN, DIRICHLET, NEUMANN, SINK, MESH, CIRCUIT
    }
  }
  return alive;
}

// Deposit of one particle with 64-bit global atomics (the slow path's particles), same
// fixed point and edge rule as the fused kernel.
template <int DOM>
__device__ inline void deposit_global_t(const MeshView& m, unsigned long long* count, long long* mom, int mom_on,
                                        const SampleView& smp, int i, int j, float fx, float fy, float wx, float wy,
                                        float vx, float vy, float vz, size_t nn, float wt = 1.f) {
  // macroparticles per cell at (int) lc (KineticMaterial.updateSamples), before the skip
  if (mom_on && smp.mpc) atomicAdd(&smp.mpc[(size_t)(j + (fy >= 1.f)) * m.ni + i + (fx >= 1.f)], 1u);
  if ((fx >= 1.f && i == m.ni - 2) || (fy >= 1.f && j == m.nj - 2)) return;  // scatter skip rule
  const size_t u = (size_t)j * m.ni + i;
  // wt: the particle's fraction of the species weight (1 without per-particle weights)
  const float s[4] = {wt * ((1.f - wx) * (1.f - wy)), wt * (wx * (1.f - wy)), wt * (wx * wy), wt * ((1.f - wx) * wy)};
  const size_t off[4] = {0, 1, (size_t)m.ni + 1, (size_t)m.ni};
  // the tile deposit's quantisation, so that a particle adds the same integers whichever
  // path finishes it
  for (int cc = 0; cc < 4; cc++) atomicAdd(&count[u + off[cc]], (unsigned long long)quant22(s[cc]) << TILE_SHIFT);
  if (mom_on) {
    const float vv[3] = {vx, vy, vz};
    for (int cc = 0; cc < 4; cc++)
      for (int dd = 0; dd < 3; dd++)
        atomicAdd((unsigned long long*)&mom[dd * nn + u + off[cc]],
                  (unsigned long long)__float2ll_rn(s[cc] * vv[dd] * 65536.0f));
    if (smp.mom2)
      for (int cc = 0; cc < 4; cc++)
        for (int dd = 0; dd < 3; dd++)
          atomicAdd(&smp.mom2[dd * nn + u + off[cc]], __float2ull_rn(s[cc] * vv[dd] * vv[dd] * (float)MOM2_SCALE));
  }
}
#define deposit_global deposit_global_t<DOM>

// The fast path's FP32 move of a particle in cell (i, j) at fraction f with the updated
// velocity nv: the new position (gx, gy) in cells relative to node (i, j), not yet
// reduced to a cell, and for RZ / ZR the velocity rotated into the new (z, r) plane
// (rotateToRZ / rotateToZR, KineticMaterial.java:424-462, relative to the cell radius).
template <int DOM>
__device__ __forceinline__ void move_fp32(int i, int j, float2 f, const PushArgs& a, float& gx, float& gy,
                                          float nv[3]) {
  if (DOM == SF_DOMAIN_XY) {
    gx = f.x + nv[0] * a.dt_dx;
    gy = f.y + nv[1] * a.dt_dy;
  } else if (DOM == SF_DOMAIN_ZR) {
    gx = f.x + nv[0] * a.dt_dx;
    const float rj = a.r0y + (float)j * a.dy;
    const float A = nv[2] * a.dt, dl = f.y * a.dy + nv[1] * a.dt;
    const float B = rj + dl, R = sqrtf(A * A + B * B), den = R + rj;
    gy = (den > 0.f ? (A * A + dl * (2.f * rj + dl)) / den : 0.f) / a.dy;
    const float cs = R > 0.f ? B / R : 1.f, sn = R > 0.f ? A / R : 0.f;
    const float v1 = nv[1], v2 = nv[2];
    nv[1] = cs * v1 + sn * v2;
    nv[2] = -sn * v1 + cs * v2;
  } else {
    gy = f.y + nv[1] * a.dt_dy;
    const float ri = a.r0x + (float)i * a.dx;
    const float A = nv[2] * a.dt, dl = f.x * a.dx + nv[0] * a.dt;
    const float B = ri + dl, R = sqrtf(A * A + B * B), den = R + ri;
    gx = (den > 0.f ? (A * A + dl * (2.f * ri + dl)) / den : 0.f) / a.dx;
    const float cs = R > 0.f ? B / R : 1.f, sn = R > 0.f ? A / R : 0.f;
    const float v1 = nv[0], v2 = nv[2];
    nv[0] = cs * v1 + sn * v2;
    nv[2] = -sn * v1 + cs * v2;
  }
}

// Conservative FP32 test of a move from (i + fx, j + fy) to (i + gx, j + gy) in cells:
// false means the path cannot meet any DIRICHLET/SINK segment listed on the nodes of
// its box (the candidate set of KineticMaterial.ProcessBoundary, :480-515), so the
// reference would find no hit.  Near-parallel or near-touching cases answer true and
// go to the exact FP64 path.
__device__ bool may_hit_fp32(const MeshView& m, int i, int j, float fx, float fy, float gx, float gy) {
  int i_min = i + (int)floorf(fminf(fx, gx)), i_max = i + (int)floorf(fmaxf(fx, gx));
  int j_min = j + (int)floorf(fminf(fy, gy)), j_max = j + (int)floorf(fmaxf(fy, gy));
  i_min = max(i_min, 0);
  j_min = max(j_min, 0);
  i_max = min(i_max, m.ni - 1);
  j_max = min(j_max, m.nj - 1);
  bool hit = false;
  for_each_candidate(m, i_min, i_max, j_min, j_max, [&](int sgi) {
    const SegLC sl = m.seg_lc[sgi];  // end points in cells relative to node (i, j)
    return hit = seg_may_cross_fp32((float)(sl.i1 - i) + sl.f1, (float)(sl.j1 - j) + sl.g1, (float)(sl.i2 - i) + sl.f2,
                                    (float)(sl.j2 - j) + sl.g2, fx, fy, gx, gy);
  });
  return hit;
}

// Every candidate segment either cannot meet the straight path (i + fx, j + fy) ->
// (i + gx, j + gy) or meets it clearly inside both parameter ranges, and the nearest of
// those crossings is clearly nearer than the next: the exact path's hit (ProcessBoundary,
// KineticMaterial.java:480-515, the smallest path parameter) is that segment.  *seg,
// *tseg: the segment and the parameter along it.
__device__ bool first_hit_fp32(const MeshView& m, int i, int j, float fx, float fy, float gx, float gy, int* seg,
                               float* tseg) {
  int i_min = i + (int)floorf(fminf(fx, gx)), i_max = i + (int)floorf(fmaxf(fx, gx));
  int j_min = j + (int)floorf(fminf(fy, gy)), j_max = j + (int)floorf(fmaxf(fy, gy));
  i_min = max(i_min, 0);
  j_min = max(j_min, 0);
  i_max = min(i_max, m.ni - 1);
  j_max = min(j_max, m.nj - 1);
  int found = -1, undecided = 0;
  float tf = 0.f, tb = 2.f, mb = 0.f, t2 = 2.f, m2 = 0.f;  // nearest crossing and the next
  for_each_candidate(m, i_min, i_max, j_min, j_max, [&](int sgi) {
    const SegLC sl = m.seg_lc[sgi];
    float ts, tp, mg;
    const int c = seg_class_fp32((float)(sl.i1 - i) + sl.f1, (float)(sl.j1 - j) + sl.g1, (float)(sl.i2 - i) + sl.f2,
                                 (float)(sl.j2 - j) + sl.g2, fx, fy, gx, gy, &ts, &tp, &mg);
    if (c == 0) return false;
    if (c == 2) {
      undecided = 1;
      return true;
    }
    if (tp < tb) {
      t2 = tb;
      m2 = mb;
      found = sgi;
      tb = tp;
      mb = mg;
      tf = ts;
    } else if (tp < t2) {
      t2 = tp;
      m2 = mg;
    }
    return false;
  });
  if (undecided || found < 0) return false;
  if (t2 < 2.f && !(t2 - tb > 2.f * (mb + m2))) return false;  // the two nearest are not clearly ordered
  *seg = found;
  *tseg = tf;
  return true;
}

// The exact path over the slow-queue entries t_first, t_first + t_stride, ... below t_end
// (every thread of the block calls it; totals are flushed to the instance at the end).
template <int DOM>
__device__ __forceinline__ void push_slow_body(const MeshView& m, const ParticlesView& P, const PushArgs& a,
                                               const SlowArgs& sg, const int* __restrict__ slow_idx,
                                               unsigned long long* __restrict__ count, long long* __restrict__ mom,
                                               int mom_on, const SampleView& smp, unsigned long long t_first,
                                               unsigned long long t_end, unsigned long long t_stride) {
  // Totals, counters and (for small geometries) per-segment surface sums are first
  // accumulated per block in shared memory and flushed once at the end: the exact
  // path's particles hit the same few segments, so global atomics would serialise.
  __shared__ double s_stats[8];
  __shared__ double s_seg[4 * SMALL_NSEG];
  __shared__ unsigned long long s_cnt[4];
  // absorptions decided in FP32 per segment: count and the sum of the segment parameter
  // in fixed point (2^-24, split in 12-bit halves: a block sees at most 2^31 / 2432
  // entries, whose sums stay below 2^32)
  __shared__ unsigned s_ahit[SMALL_NSEG], s_atlo[SMALL_NSEG], s_athi[SMALL_NSEG];
  // slow-queue entries waiting for the exact path (at most two blocks' worth: below one
  // before an iteration adds at most one)
  __shared__ int s_exact[2 * SLOW_THREADS];
  __shared__ int s_nex;
  const bool seg_local = m.nseg <= SMALL_NSEG;
  __syncthreads();  // a block calling this again: the previous call's flush has read everything
  for (int q = threadIdx.x; q < 8; q += blockDim.x) s_stats[q] = 0.0;
  for (int q = threadIdx.x; q < 4 * SMALL_NSEG; q += blockDim.x) s_seg[q] = 0.0;
  for (int q = threadIdx.x; q < SMALL_NSEG; q += blockDim.x) s_ahit[q] = s_atlo[q] = s_athi[q] = 0u;
  if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0ULL;
  if (threadIdx.x == 0) s_nex = 0;
  __syncthreads();
  SlowArgs sa = sg;
  sa.stats_slow = s_stats;
  sa.counters = s_cnt;
  if (seg_local) {
    sa.sv.flux = s_seg;
    sa.sv.deposit = s_seg + 2 * SMALL_NSEG;
  }
  const size_t nn = (size_t)m.ni * m.nj;
  // per-thread totals of the particles finished here (one shared atomic per warp at the
  // end instead of six per particle on the same few addresses)
  double lst[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  unsigned long long ldone = 0;
  unsigned nabs = 0;  // absorptions decided in FP32 (boundary charge)
  const bool want = sg.stats != 0;
  // The exact FP64 path, for one particle.
  auto exact_one = [&](int64_t p) {
    const uint32_t c = P.cell[p];
    const float2 f = P.frac[p];
    const float2 v = P.vxy[p];
    const float wp = P.w ? P.w[p] : 1.f;  // fraction of the species weight
    PushArgs ap = a;                       // the particle's own weight in the surface sums
    ap.spwt = a.spwt * (double)wp;
    double lc[2] = {cell_i(c) + (double)f.x, cell_j(c) + (double)f.y};
    double pos[2] = {m.x0[0] + lc[0] * m.dh[0], m.x0[1] + lc[1] * m.dh[1]};
    double vel[3] = {v.x, v.y, (double)P.vz[p]};
    double pdt = a.dt64;
    Philox rng(a.seed, RNG_SURFACE, (uint64_t)p, a.step);
    int bounces = 0;
    bool alive = true, periodic = false;
    while (pdt > 0 && bounces++ < 10) {
      const double old[2] = {pos[0], pos[1]};
      const double lc_old[2] = {lc[0], lc[1]};
      pos[0] += vel[0] * pdt;
      pos[1] += vel[1] * pdt;
      if (DOM == SF_DOMAIN_RZ) {
        const double A = vel[2] * pdt, B = pos[0];
        const double R = sqrt(A * A + B * B);
        const double iR = R > 0 ? 1.0 / R : 0.0;
        const double cs = R > 0 ? B * iR : 1.0, sn = R > 0 ? A * iR : 0.0;
        const double v1 = vel[0], v2 = vel[2];
        pos[0] = R;
        vel[0] = cs * v1 + sn * v2;
        vel[2] = -sn * v1 + cs * v2;
      } else if (DOM == SF_DOMAIN_ZR) {
        const double A = vel[2] * pdt, B = pos[1];
        const double R = sqrt(A * A + B * B);
        const double iR = R > 0 ? 1.0 / R : 0.0;
        const double cs = R > 0 ? B * iR : 1.0, sn = R > 0 ? A * iR : 0.0;
        const double v1 = vel[1], v2 = vel[2];
        pos[1] = R;
        vel[1] = cs * v1 + sn * v2;
        vel[2] = -sn * v1 + cs * v2;
      }
      lc[0] = (pos[0] - m.x0[0]) * m.inv_dh[0];
      lc[1] = (pos[1] - m.x0[1]) * m.inv_dh[1];
      periodic = false;
      alive = process_boundary(m, sa, ap, pos, vel, lc, pdt, old, lc_old, rng, periodic);
      if (!alive) break;
    }
    if (!alive) {
      P.cell[p] = DEAD;
      atomicAdd(&sa.counters[1], 1ULL);
      return;
    }
    if (pdt > 0) atomicAdd(&sa.counters[2], 1ULL);  // remaining time is dropped
    if (periodic) {
      lc[0] = fmin(fmax((pos[0] - m.x0[0]) * m.inv_dh[0], 0.0), m.ni - 1.0);
      lc[1] = fmin(fmax((pos[1] - m.x0[1]) * m.inv_dh[1], 0.0), m.nj - 1.0);
    }
    int i = (int)lc[0], j = (int)lc[1];
    if (i > m.ni - 2) i = m.ni - 2;
    if (j > m.nj - 2) j = m.nj - 2;
    if (i < 0) i = 0;
    if (j < 0) j = 0;
    const float fx = (float)(lc[0] - i), fy = (float)(lc[1] - j);
    P.cell[p] = pack_cell(i, j);
    P.frac[p] = make_float2(fx, fy);
    P.vxy[p] = make_float2((float)vel[0], (float)vel[1]);
    P.vz[p] = (float)vel[2];
    if (want) {
      lst[0] += (double)wp;
      lst[1] += wp * vel[0];
      lst[2] += wp * vel[1];
      lst[3] += wp * vel[2];
      lst[4] += wp * sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    }
    float wx, wy;
    scatter_weights<DOM>(fx, fy, i, j, a, wx, wy);
    deposit_global(m, count, mom, mom_on, smp, i, j, fx, fy, wx, wy, (float)vel[0], (float)vel[1], (float)vel[2], nn,
                   wp);
  };
  // The FP32 pre-filter, for one particle: true when it has to take the exact path.
  auto prefilter = [&](int64_t p) -> bool {
    const uint32_t c = P.cell[p];
    const float2 f = P.frac[p];
    const float2 v = P.vxy[p];
    const float wp = P.w ? P.w[p] : 1.f;
    // a particle whose (logical, straight) path certainly misses every candidate segment
    // and stays in the mesh finishes exactly like the fast path
    const int i = cell_i(c), j = cell_j(c);
    float gx, gy, nv[3] = {v.x, v.y, P.vz[p]};
    move_fp32<DOM>(i, j, f, a, gx, gy, nv);
    if (!may_hit_fp32(m, i, j, f.x, f.y, gx, gy)) {
      float fdi = floorf(gx), fdj = floorf(gy);
      float nfx = gx - fdi, nfy = gy - fdj;
      if (nfx >= 1.f) { nfx -= 1.f; fdi += 1.f; }
      if (nfy >= 1.f) { nfy -= 1.f; fdj += 1.f; }
      const int i2 = i + (int)fdi, j2 = j + (int)fdj;
      const bool inside = (i2 >= 0) & (j2 >= 0) & (i2 <= m.ni - 2) & (j2 <= m.nj - 2);
      if (inside) {
        P.cell[p] = pack_cell(i2, j2);
        P.frac[p] = make_float2(nfx, nfy);
        if (DOM != SF_DOMAIN_XY) {  // the rotation changed the velocity
          P.vxy[p] = make_float2(nv[0], nv[1]);
          P.vz[p] = nv[2];
        }
        ldone++;
        if (want) {
          lst[0] += (double)wp;
          lst[1] += (double)(wp * nv[0]);
          lst[2] += (double)(wp * nv[1]);
          lst[3] += (double)(wp * nv[2]);
          lst[4] += (double)(wp * sqrtf(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]));
        }
        float wx, wy;
        scatter_weights<DOM>(nfx, nfy, i2, j2, a, wx, wy);
        deposit_global(m, count, mom, mom_on, smp, i2, j2, nfx, nfy, wx, wy, nv[0], nv[1], nv[2], nn, wp);
        return false;
      }
      if (m.all_delete) {
        P.cell[p] = DEAD;
        atomicAdd(&sa.counters[1], 1ULL);
        atomicAdd(&sa.counters[3], 1ULL);
        return false;
      }
      return true;
    }
    // a clear first hit of an absorbing segment (the common case of ions striking an
    // electrode): the exact path would take the same segment and remove the particle
    // there; only the flux and deposit shares need the hit point
    int hs;
    float ht;
    if (!P.w && first_hit_fp32(m, i, j, f.x, f.y, gx, gy, &hs, &ht)) {
      const int model = sa.sv.model[hs];
      if (model != SF_SURF_PASS && model != SF_SURF_NONE && model != SF_SURF_SPECULAR &&
          model != SF_SURF_DIFFUSE) {
        nabs++;
        if (seg_local) {
          const unsigned qt = __float2uint_rn(ht * 16777216.f);
          atomicAdd(&s_ahit[hs], 1u);
          atomicAdd(&s_atlo[hs], qt & 0xFFFu);
          atomicAdd(&s_athi[hs], qt >> 12);
        } else {
          const double w1 = a.spwt * (1 - (double)ht), w2 = a.spwt * (double)ht;
          atomicAdd(&sa.sv.flux[2 * hs], w1);
          atomicAdd(&sa.sv.flux[2 * hs + 1], w2);
          atomicAdd(&sa.sv.deposit[2 * hs], w1);
          atomicAdd(&sa.sv.deposit[2 * hs + 1], w2);
        }
        P.cell[p] = DEAD;
        atomicAdd(&sa.counters[1], 1ULL);
        return false;
      }
    }
    return true;
  };
  // Particles that need the exact path are gathered in a block-local list and run by
  // consecutive threads once a block's worth is there (and at the end), so that the FP64
  // work runs in full warps instead of one or two lanes of every warp.  The entries
  // t_first - threadIdx.x + k t_stride are the same for the whole block.
  const int nb = blockDim.x;
  for (unsigned long long t0 = t_first - threadIdx.x; t0 < t_end; t0 += t_stride) {
    const unsigned long long t = t0 + threadIdx.x;
    const bool ex = t < t_end && prefilter(slow_idx[t]);
    const unsigned mex = __ballot_sync(0xffffffffu, ex);
    if (mex) {
      const int leader = __ffs(mex) - 1;
      int base = 0;
      if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(&s_nex, __popc(mex));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (ex) s_exact[base + __popc(mex & ((1u << (threadIdx.x & 31)) - 1u))] = (int)slow_idx[t];
    }
    __syncthreads();
    const int nex = s_nex;
    if (nex >= nb) {
      const int q = s_exact[nex - nb + threadIdx.x];
      __syncthreads();  // every entry read before the list shrinks and refills
      if (threadIdx.x == 0) s_nex = nex - nb;
      exact_one(q);
      __syncthreads();
    }
  }
  {
    const int nex = s_nex;
    if ((int)threadIdx.x < nex) exact_one(s_exact[threadIdx.x]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    if (want)
      for (int q = 0; q < 5; q++) lst[q] += __shfl_down_sync(0xffffffffu, lst[q], o);
    ldone += __shfl_down_sync(0xffffffffu, ldone, o);
    nabs += __shfl_down_sync(0xffffffffu, nabs, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (want) {
      for (int q = 0; q < 5; q++)
        if (lst[q] != 0.0) atomicAdd(&s_stats[q], lst[q]);
      if (nabs) atomicAdd(&s_stats[5], (double)nabs * (a.spwt * a.charge));
    }
    if (ldone) atomicAdd(&s_cnt[3], ldone);
  }
  __syncthreads();
  // FP32-decided absorptions into the per-segment sums: N hits with parameters t sum to
  // spwt (N - sum t) at the first end and spwt sum t at the second (flux and deposit)
  if (seg_local) {
    for (int q = threadIdx.x; q < m.nseg; q += blockDim.x)
      if (s_ahit[q]) {
        const double T = ((double)s_athi[q] * 4096.0 + (double)s_atlo[q]) * (1.0 / 16777216.0);
        const double w1 = a.spwt * ((double)s_ahit[q] - T), w2 = a.spwt * T;
        s_seg[2 * q] += w1;
        s_seg[2 * q + 1] += w2;
        s_seg[2 * SMALL_NSEG + 2 * q] += w1;
        s_seg[2 * SMALL_NSEG + 2 * q + 1] += w2;
      }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < 6; q += blockDim.x)
    if (s_stats[q] != 0.0) atomicAdd(&sg.stats_slow[q], s_stats[q]);
  if (threadIdx.x >= 1 && threadIdx.x < 4 && s_cnt[threadIdx.x])
    atomicAdd(&sg.counters[threadIdx.x], s_cnt[threadIdx.x]);
  if (seg_local)
    for (int q = threadIdx.x; q < 2 * m.nseg; q += blockDim.x) {
      if (s_seg[q] != 0.0) atomicAdd(&sg.sv.flux[q], s_seg[q]);
      if (s_seg[2 * SMALL_NSEG + q] != 0.0) atomicAdd(&sg.sv.deposit[q], s_seg[2 * SMALL_NSEG + q]);
    }
}

template <int DOM>
__global__ void __launch_bounds__(SLOW_THREADS) k_push_slow(MeshView m, ParticlesView P, PushArgs a, SlowArgs sg,
                                                   const int* __restrict__ slow_idx,
                                                   unsigned long long* __restrict__ count,
                                                   long long* __restrict__ mom, int mom_on, SampleView smp) {
  push_slow_body<DOM>(m, P, a, sg, slow_idx, count, mom, mom_on, smp,
                     (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x, sg.counters[0],
                     (unsigned long long)gridDim.x * blockDim.x);
}

// Node density from the fixed-point count: count x (spwt / 2^31 / V, the species' factor
// computed once on the host) + nd_back.  Dividing by the volume here made this epilogue
// FP64-bound (an FP64 divide is a dozen FP64-pipe instructions).
__device__ __forceinline__ double node_density(unsigned long long c, double factor, double nd_back) {
  return fma((double)c, factor, nd_back);
}

// int64 fixed point -> density (Field2D.scaleByVol, Field2D.java:418-431) and mean
// velocities (Field2D.divideByField, :403-414)
// Thread 0 also keeps the species' push counters: live_base = slots - removed slots
// the host knows of, so live_base - acc[0] particles were alive when this push began.
__global__ void k_finalize(int nn, const unsigned long long* __restrict__ count, const long long* __restrict__ mom,
                           const double* __restrict__ nd_factor, double nd_back,
                           double* __restrict__ nd, double* __restrict__ uvw, int mom_on,
                           unsigned long long* __restrict__ acc, const unsigned long long* __restrict__ counters,
                           long long live_base) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned long long removed_before = acc[0];
    acc[1] += (unsigned long long)(live_base - (long long)removed_before);
    acc[0] = removed_before + counters[1];
  }
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nn; u += gridDim.x * blockDim.x) {
    const unsigned long long c = count[u];
    nd[u] = node_density(c, nd_factor[u], nd_back);
    if (mom_on) {
      for (int d = 0; d < 3; d++)
        uvw[(size_t)d * nn + u] = c ? ((double)mom[(size_t)d * nn + u] / MOM_SCALE) / ((double)c / DEP_SCALE) : 0.0;
    }
  }
}

// running sums of the velocity sampling (KineticMaterial.updateSamples,
// KineticMaterial.java:1570-1595): count, u, v, w, uu, vv, ww (scattered w S v^k, in
// weight units) and mpc.  The per-step values are exact integer sums, added in step
// order, so the sums are reproducible.
__global__ void k_sample_accum(int nn, const unsigned long long* __restrict__ count, const long long* __restrict__ mom,
                               const unsigned long long* __restrict__ mom2, const unsigned* __restrict__ mpc,
                               double spwt, double* __restrict__ samp) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nn; u += gridDim.x * blockDim.x) {
    samp[u] += (double)count[u] * (spwt / DEP_SCALE);
    for (int d = 0; d < 3; d++) {
      samp[(size_t)(1 + d) * nn + u] += (double)mom[(size_t)d * nn + u] * (spwt / MOM_SCALE);
      samp[(size_t)(4 + d) * nn + u] += (double)mom2[(size_t)d * nn + u] * (spwt / MOM2_SCALE);
    }
    samp[(size_t)7 * nn + u] += (double)mpc[u];
  }
}

// KineticMaterial.computeFields (KineticMaterial.java:1606-1671): temperatures from the
// sampled moments (the initial temperature where nothing was sampled), averaged density
// (count / samples / node volume), mean velocities, pressure n k T, particles per cell
__global__ void k_gas_fields(int nn, const double* __restrict__ samp, double inv_samples, const double* __restrict__ vol,
                             double m_over_k, double T_init, double* __restrict__ gas) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nn; u += gridDim.x * blockDim.x) {
    const double c = samp[u];
    double T = T_init, T1 = T_init, T2 = T_init, T3 = T_init, U[3] = {0, 0, 0};
    if (c > 0) {
      double uu[3];
      for (int d = 0; d < 3; d++) {
        U[d] = samp[(size_t)(1 + d) * nn + u] / c;
        uu[d] = samp[(size_t)(4 + d) * nn + u] / c - U[d] * U[d];
      }
      T = (uu[0] + uu[1] + uu[2]) * m_over_k / 3.0;
      T1 = uu[0] * m_over_k;
      T2 = uu[1] * m_over_k;
      T3 = uu[2] * m_over_k;
    }
    const double nd = c * inv_samples / vol[u];
    gas[u] = nd;
    for (int d = 0; d < 3; d++) gas[(size_t)(1 + d) * nn + u] = U[d];
    gas[(size_t)4 * nn + u] = T;
    gas[(size_t)5 * nn + u] = T1;
    gas[(size_t)6 * nn + u] = T2;
    gas[(size_t)7 * nn + u] = T3;
    gas[(size_t)8 * nn + u] = nd * KB * T;
    gas[(size_t)9 * nn + u] = samp[(size_t)7 * nn + u] * inv_samples;
  }
}

// deterministic sum of the per-block partials: one warp per quantity, lanes take fixed
// strided subsets and a fixed shuffle tree combines them
__global__ void k_sum_partials(const double* part, int nblocks, double* out) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (q >= 5) return;
  double s = 0;
  for (int b = lane; b < nblocks; b += 32) s += part[(size_t)b * 8 + q];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[q] = s;
}

// Per-call scratch of one push: the slow-path queue (one slot per particle), the event
// counters, the per-block partial sums (stats_blocks x 8 doubles, the last row holds the
// slow-path sums) and the 8-double output of k_sum_partials.
struct PushScratch {
  int* slow_idx;
  unsigned long long* counters;
  double* stats_partial;
  int stats_blocks;
  double* sums;
};

// ---------------------------------------------------------------------------------
// batched push over the instances of a batch (one launch for all instances)
// ---------------------------------------------------------------------------------
// instance holding global tile gt: tile_start[i] <= gt < tile_start[i + 1]
__device__ __forceinline__ int batch_find(const int64_t* __restrict__ tile_start, int n, int64_t gt) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (tile_start[mid] <= gt) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Exclusive prefix of val(0..n-1) into out[0..n] (out[n] = total) by one block whose size
// is a multiple of 32; val(i) is called once per i.
template <typename F>
__device__ void block_exclusive_prefix(int n, F val, int64_t* __restrict__ out) {
  __shared__ int64_t wsum[32];
  __shared__ int64_t carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int64_t v = i < n ? val(i) : 0;
    int64_t x = v;  // inclusive prefix within the warp
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int64_t w = lane < nwarps ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;  // inclusive prefix of the warp totals
    }
    __syncthreads();
    const int64_t before = carry + (warp > 0 ? wsum[warp - 1] : 0) + x - v;
    if (i < n) out[i] = before;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// slots in use after this step's injection, and the prefix of push tiles (one block)
__global__ void __launch_bounds__(1024) k_batch_begin(BatchDev b) {
  block_exclusive_prefix(
      b.n,
      [&](int i) {
        const int64_t nd = b.base_dev[i] + (int64_t)b.added_dev[i];
        b.n_dev[i] = nd;
        return (nd + TILE - 1) / TILE;
      },
      b.tile_start);
}

// the slow queues of all instances cut into chunks of SLOW_CHUNK entries: prefix of the
// chunk counts (one block, after the batched fast push filled the queues)
constexpr int SLOW_CHUNK = 512;
__global__ void __launch_bounds__(1024) k_slow_plan(BatchDev b) {
  block_exclusive_prefix(
      b.n, [&](int i) { return (int64_t)((b.insts[i].sa.counters[0] + SLOW_CHUNK - 1) / SLOW_CHUNK); },
      b.chunk_start);
}

// per instance: zero the deposit, the push counters and the slow-path sums
__global__ void k_batch_zero(BatchDev b) {
  const BatchInst& I = b.insts[blockIdx.y];
  const int nn = I.m.ni * I.m.nj;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nn; u += gridDim.x * blockDim.x) I.count[u] = 0ULL;
  if (blockIdx.x == 0 && threadIdx.x < 8) {
    if (threadIdx.x < 4) I.sa.counters[threadIdx.x] = 0ULL;
    I.sa.stats_slow[threadIdx.x] = 0.0;
  }
}

// 4 blocks of PB per SM (64 registers, with spills): in the batched step faster than 2
// blocks (123 registers) or 3 (80).  W: some instance's species carries per-particle
// weights (the others read as weight 1)
template <int DOM, bool W>
__global__ void __launch_bounds__(PB, 4) k_push_batch(BatchDev b) {
  __shared__ unsigned acc[SBOX];
  __shared__ int sred[4][PB / 32];
  Kahan st_px, st_py, st_pz, st_e;
  unsigned st_n = 0;
  for (int q = threadIdx.x; q < SBOX; q += PB) acc[q] = 0u;
  __syncthreads();
  const int64_t total = b.tile_start[b.n];
  for (int64_t gt = blockIdx.x; gt < total; gt += gridDim.x) {
    const int i = batch_find(b.tile_start, b.n, gt);
    const BatchInst& I = b.insts[i];
    ParticlesView P = I.P;
    P.n = b.n_dev[i];
    push_tile<DOM, false, false, true, W>(I.m, P, I.a, (gt - b.tile_start[i]) * TILE, I.count, nullptr, I.slow_idx,
                                 I.sa.counters, SampleView{nullptr, nullptr}, acc, sred, st_px, st_py,
                                 st_pz, st_e, st_n, st_e);
  }
}

// The exact path over the chunks of all instances' slow queues: every block takes chunks
// in turn, so an instance with a long queue is spread over the whole GPU.
template <int DOM>
__global__ void __launch_bounds__(SLOW_THREADS) k_push_slow_batch(BatchDev b) {
  const int64_t total = b.chunk_start[b.n];
  for (int64_t c = blockIdx.x; c < total; c += gridDim.x) {
    const int i = batch_find(b.chunk_start, b.n, c);
    const BatchInst& I = b.insts[i];
    const unsigned long long t0 = (unsigned long long)(c - b.chunk_start[i]) * SLOW_CHUNK;
    const unsigned long long t1 = min(t0 + (unsigned long long)SLOW_CHUNK, I.sa.counters[0]);
    push_slow_body<DOM>(I.m, I.P, I.a, I.sa, I.slow_idx, I.count, nullptr, 0, SampleView{nullptr, nullptr},
                        t0 + threadIdx.x, t1, blockDim.x);
  }
}

// nd = count w / V + nd_back per instance; removed slots counted; the instance's push
// step (its surface RNG epoch) and the batch step advanced
__global__ void k_finalize_batch(BatchDev b) {
  BatchInst& I = b.insts[blockIdx.y];
  const int nn = I.m.ni * I.m.nj;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nn; u += gridDim.x * blockDim.x)
    I.nd[u] = node_density(I.count[u], I.nd_factor[u], I.nd_back);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    b.dead_dev[blockIdx.y] += (int64_t)I.sa.counters[1];
    I.a.step++;
    if (blockIdx.y == 0) atomicAdd(b.step_dev, 1u);
  }
}

template <int DOM, bool STATS, bool MOM>
void launch_push_t(sf_ctx* ctx, SfSpecies* sp, const PushArgs& a, int grid, const PushScratch& sc,
                   const SampleView& smp) {
  if (sp->cur.w)
    k_push<DOM, STATS, MOM, true><<<grid, PB, 0, ctx->stream>>>(ctx->mesh_view(), sp->cur, a, sp->count, sp->mom,
                                                                sc.slow_idx, sc.counters, sc.stats_partial, smp);
  else
    k_push<DOM, STATS, MOM, false><<<grid, PB, 0, ctx->stream>>>(ctx->mesh_view(), sp->cur, a, sp->count, sp->mom,
                                                                 sc.slow_idx, sc.counters, sc.stats_partial, smp);
}

template <int DOM>
void launch_push_dom(sf_ctx* ctx, SfSpecies* sp, const PushArgs& a, int grid, bool stats, bool mom,
                     const PushScratch& sc, const SampleView& smp) {
  if (stats && mom) launch_push_t<DOM, true, true>(ctx, sp, a, grid, sc, smp);
  else if (stats) launch_push_t<DOM, true, false>(ctx, sp, a, grid, sc, smp);
  else if (mom) launch_push_t<DOM, false, true>(ctx, sp, a, grid, sc, smp);
  else launch_push_t<DOM, false, false>(ctx, sp, a, grid, sc, smp);
}

}  // namespace

namespace sf {

void batch_push(const BatchDev& b, cudaStream_t stream, int num_sms, int blocks_per_sm, int slow_blocks_per_sm) {
  k_batch_begin<<<1, 1024, 0, stream>>>(b);
  k_batch_zero<<<dim3(8, b.n), 256, 0, stream>>>(b);
  if (b.any_weighted)
    k_push_batch<SF_DOMAIN_XY, true><<<num_sms * blocks_per_sm, PB, 0, stream>>>(b);
  else
    k_push_batch<SF_DOMAIN_XY, false><<<num_sms * blocks_per_sm, PB, 0, stream>>>(b);
  k_slow_plan<<<1, 1024, 0, stream>>>(b);
  k_push_slow_batch<SF_DOMAIN_XY><<<num_sms * slow_blocks_per_sm, SLOW_THREADS, 0, stream>>>(b);
  k_finalize_batch<<<dim3(4, b.n), 256, 0, stream>>>(b);
  SF_CUDA(cudaGetLastError());
}

void launch_finalize(sf_ctx* ctx, SfSpecies* sp, bool moments, const unsigned long long* counters) {
  int nn = ctx->ni * ctx->nj;
  ctx->launches++;
  k_finalize<<<grid_for(nn, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      nn, sp->count, sp->mom, sp->nd_factor, sp->nd_back, sp->nd, sp->uvw, moments ? 1 : 0,
      sp->acc, counters, (long long)(sp->n - sp->n_dead));
}

}  // namespace sf

namespace {

// Body of sf_push_deposit and sf_push_deposit_noalloc: they differ only in where the
// per-call scratch lives.  Allocates nothing.
void push_deposit_impl(sf_ctx* ctx, SfSpecies* sp, double dt, int32_t flags, sf_push_stats* stats,
                       const PushScratch& sc) {
  const bool want_stats = (flags & SF_PUSH_STATS) != 0;
  const bool sample = (flags & SF_PUSH_SAMPLE) != 0;
  const bool mom = sample || (flags & SF_PUSH_MOMENTS) != 0;
  // totals and surface products need the host to read this push's results
  const bool nowait = (flags & SF_PUSH_NOWAIT) != 0 && !want_stats && !sp->has_products;
  SF_REQUIRE(!sample || sp->samp, SF_ERR_STATE, "velocity sampling not set up (sf_samples_clear)");
  const SampleView smp = sample ? sp->smp : SampleView{nullptr, nullptr};
  // automatic sort every sort_interval pushes (the counter starts at the interval, so the
  // first push of a species sorts); the key looks half an interval ahead, so that the
  // tiles are most compact in the middle of the interval, and is that of the species'
  // sort block of cells (locality only)
  if (sp->sort_interval > 0 && sp->pushes_since_sort >= sp->sort_interval) {
    const double tau = 0.5 * sp->sort_interval * dt;
    launch_sort(ctx, sp, (float)(tau / ctx->dh[0]), (float)(tau / ctx->dh[1]), sp->sort_qb);
  }
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  cudaStream_t s = ctx->stream;
  SF_CUDA(cudaMemsetAsync(sp->count, 0, sizeof(unsigned long long) * nn, s));
  if (mom) SF_CUDA(cudaMemsetAsync(sp->mom, 0, sizeof(long long) * 3 * nn, s));
  if (sample) {
    SF_CUDA(cudaMemsetAsync(smp.mom2, 0, sizeof(unsigned long long) * 3 * nn, s));
    SF_CUDA(cudaMemsetAsync(smp.mpc, 0, sizeof(unsigned) * nn, s));
  }
  SF_CUDA(cudaMemsetAsync(sc.counters, 0, sizeof(unsigned long long) * 8, s));
  // stats_partial tail (after the per-block area) holds the slow-path sums
  double* slow_stats = sc.stats_partial + (size_t)8 * (sc.stats_blocks - 1);
  if (want_stats) SF_CUDA(cudaMemsetAsync(sc.stats_partial, 0, sizeof(double) * 8 * (size_t)sc.stats_blocks, s));

  PushArgs a;
  a.qm_dt = (float)(sp->charge / sp->mass * dt);
  a.dt_dx = (float)(dt / ctx->dh[0]);
  a.dt_dy = (float)(dt / ctx->dh[1]);
  a.dt = (float)dt;
  a.dx = (float)ctx->dh[0];
  a.dy = (float)ctx->dh[1];
  a.r0x = (float)ctx->x0[0];
  a.r0y = (float)ctx->x0[1];
  a.dt64 = dt;
  a.qm = sp->charge / sp->mass;
  a.charge = sp->charge;
  a.spwt = sp->spwt;
  a.seed = ctx->seed;
  a.step = sp->step;

  int tiles = (int)((sp->n + TILE - 1) / TILE);
  int grid = std::max(1, std::min(tiles, sc.stats_blocks - 1));
  if (sp->n > 0) {
    {
    TimedScope ts(ctx, "push");
    ctx->launches++;
    switch (ctx->domain) {
      case SF_DOMAIN_XY: launch_push_dom<SF_DOMAIN_XY>(ctx, sp, a, grid, want_stats, mom, sc, smp); break;
      case SF_DOMAIN_RZ: launch_push_dom<SF_DOMAIN_RZ>(ctx, sp, a, grid, want_stats, mom, sc, smp); break;
      default: launch_push_dom<SF_DOMAIN_ZR>(ctx, sp, a, grid, want_stats, mom, sc, smp); break;
    }
    }
    SF_CUDA(cudaGetLastError());
    SlowArgs sa;
    sa.sv.model = sp->seg_model;
    sa.sv.param = sp->seg_param;
    sa.sv.flux = sp->flux;
    sa.sv.deposit = sp->deposit;
    sa.counters = sc.counters;
    sa.stats_slow = slow_stats;
    sa.stats = want_stats ? 1 : 0;
    sa.sv.product = nullptr;
    sa.sv.prod = nullptr;
    if (sp->has_products) {
      // the species' current views (the sort swaps buffers) and zeroed append counters
      std::vector<ProductView> pv(ctx->species.size());
      for (size_t q = 0; q < pv.size(); q++) {
        const SfSpecies* o = ctx->species[q];
        pv[q].P = o->cur;
        pv[q].P.n = o->n;
        pv[q].cap = o->cap;
        pv[q].added = ctx->d_prod_added + q;
        pv[q].spwt = o->spwt;
        pv[q].qm_halfdt = (float)(o->charge / o->mass * 0.5 * dt);
        pv[q].vth = 0.f;
      }
      SF_CUDA(cudaMemcpyAsync(ctx->d_prod, pv.data(), sizeof(ProductView) * pv.size(), cudaMemcpyHostToDevice, s));
      SF_CUDA(cudaMemsetAsync(ctx->d_prod_added, 0, sizeof(unsigned long long) * pv.size(), s));
      sa.sv.product = sp->seg_product;
      sa.sv.prod = ctx->d_prod;
    }
    // 4 blocks of 128 per SM: the queue (0.2-0.5 M particles per step at 64 M ions) is
    // spread over all SMs, and each block's set-up and flush are paid fewer times
    // (0.044 -> 0.040 ms against 16 blocks per SM)
    const int sgrid = ctx->num_sms * 4;
    TimedScope ts(ctx, "push_slow");
    ctx->launches++;
    switch (ctx->domain) {
      case SF_DOMAIN_XY:
        k_push_slow<SF_DOMAIN_XY><<<sgrid, SLOW_THREADS, 0, s>>>(ctx->mesh_view(), sp->cur, a, sa, sc.slow_idx, sp->count, sp->mom, mom,
                                                        smp);
        break;
      case SF_DOMAIN_RZ:
        k_push_slow<SF_DOMAIN_RZ><<<sgrid, SLOW_THREADS, 0, s>>>(ctx->mesh_view(), sp->cur, a, sa, sc.slow_idx, sp->count, sp->mom, mom,
                                                        smp);
        break;
      default:
        k_push_slow<SF_DOMAIN_ZR><<<sgrid, SLOW_THREADS, 0, s>>>(ctx->mesh_view(), sp->cur, a, sa, sc.slow_idx, sp->count, sp->mom, mom,
                                                        smp);
        break;
    }
    SF_CUDA(cudaGetLastError());
  }
  {
    TimedScope ts(ctx, "finalize");
    launch_finalize(ctx, sp, mom, sc.counters);
  }
  if (sample) {
    // KineticMaterial.updateSamples: this step's deposits into the running sums
    TimedScope ts(ctx, "sample");
    k_sample_accum<<<grid_for((int64_t)nn, 256, ctx->num_sms * 8), 256, 0, s>>>(
        (int)nn, sp->count, sp->mom, smp.mom2, smp.mpc, sp->spwt, sp->samp);
    ctx->launches++;
    sp->num_samples++;
  }
  SF_CUDA(cudaGetLastError());
  if (nowait) {
    // the removed-slot count stays on the device (acc[0]) until a call needs it
    sp->acc_pending = true;
    sp->step++;
    sp->pushes_since_sort++;
    sp->moments_valid = mom;
    if (stats) {
      memset(stats, 0, sizeof(*stats));
      stats->np = stats->n_removed = stats->n_slow = stats->n_bounce_limited = -1;
    }
    return;
  }
  double* h = ctx->host_pinned;
  unsigned long long hc[4], removed = 0;
  SF_CUDA(cudaMemcpyAsync(hc, sc.counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
  SF_CUDA(cudaMemcpyAsync(&removed, sp->acc, sizeof(removed), cudaMemcpyDeviceToHost, s));
  SF_CUDA(cudaMemsetAsync(sp->acc, 0, sizeof(unsigned long long), s));
  if (want_stats) {
    k_sum_partials<<<1, 160, 0, s>>>(sc.stats_partial, grid, sc.sums);
    ctx->launches++;
    SF_CUDA(cudaMemcpyAsync(h, sc.sums, sizeof(double) * 5, cudaMemcpyDeviceToHost, s));
    SF_CUDA(cudaMemcpyAsync(h + 8, slow_stats, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
  }
  SF_CUDA(cudaStreamSynchronize(s));
  timer_collect(ctx);
  // this push's removals and those of earlier pushes that did not wait
  sp->n_dead += (int64_t)removed;
  sp->acc_pending = false;
  if (sp->has_products) {
    // product particles appended by surface impacts
    std::vector<unsigned long long> added(ctx->species.size());
    copy_wait(added.data(), ctx->d_prod_added, sizeof(unsigned long long) * added.size(), cudaMemcpyDeviceToHost, s);
    bool over = false;
    for (size_t q = 0; q < added.size(); q++) {
      SfSpecies* o = ctx->species[q];
      const int64_t room = o->cap - o->n;
      const int64_t k = std::min<int64_t>((int64_t)added[q], room);
      over |= (int64_t)added[q] > room;
      if (k > 0) {
        o->n += k;
        o->cur.n = o->n;
        o->sorted = false;
      }
    }
    SF_REQUIRE(!over, SF_ERR_OOM, "surface products exceeded a species' capacity (the excess was dropped)");
  }
  sp->step++;
  sp->pushes_since_sort++;
  sp->moments_valid = mom;
  if (removed > 0) sp->sorted = false;
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    if (want_stats) {
      stats->n_sum = (h[0] + h[8]) * sp->spwt;
      for (int d = 0; d < 3; d++) stats->p_sum[d] = (h[1 + d] + h[9 + d]) * sp->spwt;
      stats->e_sum = (h[4] + h[12]) * sp->spwt;
      stats->boundary_charge = h[13];
    }
    stats->np = sp->n - sp->n_dead;
    stats->n_removed = (int64_t)hc[1];
    stats->n_slow = (int64_t)hc[0];
    stats->n_bounce_limited = (int64_t)hc[2];
  }
}

// ---------------------------------------------------------------------------------
// Push scratch that needs no allocation.
//
// Some hosts cannot let the library call cudaMalloc while they step the particles: a
// host whose own caching allocator (PyTorch's, a JVM-side pool) has already reserved
// the device memory, where a stray cudaMalloc can fail or force that allocator to give
// its cache back, and services that fix their device footprint at start-up and treat
// any later allocation as a fault.  For them, the per-call scratch of the push lives in
// a file-scope __device__ array that is part of the loaded module, so it exists as soon
// as the library is on the device.
// ---------------------------------------------------------------------------------
constexpr int64_t NOALLOC_MAX_PARTICLES = int64_t(1) << 21;  // slow-queue slots (8 MiB)
constexpr int NOALLOC_MAX_STATS_BLOCKS = 4096;                // partial-sum rows (256 KiB)
constexpr size_t NOALLOC_OFF_COUNTERS = 0;
constexpr size_t NOALLOC_OFF_SUMS = 256;
constexpr size_t NOALLOC_OFF_PARTIAL = 512;
constexpr size_t NOALLOC_OFF_SLOW = NOALLOC_OFF_PARTIAL + sizeof(double) * 8 * NOALLOC_MAX_STATS_BLOCKS;
constexpr size_t NOALLOC_BYTES = NOALLOC_OFF_SLOW + sizeof(int) * NOALLOC_MAX_PARTICLES;
static_assert(NOALLOC_OFF_SLOW % 256 == 0, "scratch regions stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_push_scratch[NOALLOC_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_base[NOALLOC_MAX_DEVICES] = {};

// Device address of g_push_scratch on ctx->device, looked up once per device (the
// device must be current) and kept for the life of the process.  A host that resets a
// device (cudaDeviceReset) discards the module and with it this array, so the kept
// address is stale afterwards: such a host must not call sf_push_deposit_noalloc again
// in the same process.
unsigned char* noalloc_scratch(sf_ctx* ctx) {
  SF_REQUIRE(ctx->device >= 0 && ctx->device < NOALLOC_MAX_DEVICES, SF_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  unsigned char*& base = g_noalloc_base[ctx->device];
  if (!base) {
    void* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&p, g_push_scratch);
    if (rc != cudaSuccess || !p)
      throw Error(SF_ERR_CUDA, std::string("cudaGetSymbolAddress(push scratch) failed: ") + cudaGetErrorString(rc));
    base = static_cast<unsigned char*>(p);
  }
  return base;
}

}  // namespace

extern "C" int sf_push_deposit(sf_ctx* ctx, int32_t sid, double dt, int32_t flags, sf_push_stats* stats) {
  SF_API_BEGIN
  SfSpecies* sp = get_species_nowait(ctx, sid);
  SF_REQUIRE(dt > 0, SF_ERR_ARG, "dt must be positive");
  SF_REQUIRE(ctx->efield_set, SF_ERR_STATE, "electric field not set (sf_set_efield or a Poisson solve)");
  SF_CUDA(cudaSetDevice(ctx->device));
  const PushScratch sc{ctx->slow_idx, ctx->counters, ctx->stats_partial, ctx->stats_blocks, ctx->dscratch};
  push_deposit_impl(ctx, sp, dt, flags, stats, sc);
  SF_API_END(ctx)
}

extern "C" int sf_push_deposit_noalloc(sf_ctx* ctx, int32_t sid, double dt, int32_t flags, sf_push_stats* stats) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(dt > 0, SF_ERR_ARG, "dt must be positive");
  SF_REQUIRE(ctx->efield_set, SF_ERR_STATE, "electric field not set (sf_set_efield or a Poisson solve)");
  SF_REQUIRE(!(flags & SF_PUSH_NOWAIT), SF_ERR_ARG,
             "sf_push_deposit_noalloc waits for every call: its scratch is shared by all contexts on the device");
  SF_REQUIRE(sp->n <= NOALLOC_MAX_PARTICLES, SF_ERR_ARG,
             "sf_push_deposit_noalloc: species holds " + std::to_string(sp->n) + " particle slots, more than its " +
                 std::to_string(NOALLOC_MAX_PARTICLES) + "-particle static scratch; use sf_push_deposit");
  SF_REQUIRE(ctx->stats_blocks <= NOALLOC_MAX_STATS_BLOCKS, SF_ERR_ARG,
             "sf_push_deposit_noalloc: device has too many SMs for the static partial-sum scratch");
  SF_CUDA(cudaSetDevice(ctx->device));
  unsigned char* base = noalloc_scratch(ctx);
  // counters and partial sums are cleared by push_deposit_impl on every call; the slow
  // queue is written before it is read, so it may keep the previous call's contents
  const PushScratch sc{reinterpret_cast<int*>(base + NOALLOC_OFF_SLOW),
                       reinterpret_cast<unsigned long long*>(base + NOALLOC_OFF_COUNTERS),
                       reinterpret_cast<double*>(base + NOALLOC_OFF_PARTIAL), ctx->stats_blocks,
                       reinterpret_cast<double*>(base + NOALLOC_OFF_SUMS)};
  push_deposit_impl(ctx, sp, dt, flags, stats, sc);
  SF_API_END(ctx)
}

extern "C" int sf_species_particle_steps(sf_ctx* ctx, int32_t sid, int64_t* particle_steps) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(particle_steps, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaSetDevice(ctx->device));
  unsigned long long v = 0;
  copy_wait(&v, sp->acc + 1, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream);
  *particle_steps = (int64_t)v;
  SF_API_END(ctx)
}

extern "C" int sf_species_set_sort_interval(sf_ctx* ctx, int32_t sid, int32_t interval) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(interval >= 0, SF_ERR_ARG, "interval must be >= 0");
  sp->sort_interval = interval;
  SF_API_END(ctx)
}

extern "C" int sf_species_set_sort_block(sf_ctx* ctx, int32_t sid, int32_t cells) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  int qb = -1;
  for (int q = 0; q <= 4; q++)
    if (cells == (1 << q)) qb = q;
  SF_REQUIRE(qb >= 0, SF_ERR_ARG, "sort block must be 1, 2, 4, 8 or 16 cells");
  sp->sort_qb = qb;
  SF_API_END(ctx)
}

// KineticMaterial.clearSamples (KineticMaterial.java:1509-1530); the first call sets up
// the sampling buffers of the species (8 + 10 FP64 node fields and the per-step deposits)
extern "C" int sf_samples_clear(sf_ctx* ctx, int32_t sid) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_CUDA(cudaSetDevice(ctx->device));
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  if (!sp->samp) {
    SF_CUDA(cudaMalloc(&sp->smp.mom2, sizeof(unsigned long long) * 3 * nn));
    SF_CUDA(cudaMalloc(&sp->smp.mpc, sizeof(unsigned) * nn));
    SF_CUDA(cudaMalloc(&sp->gas, sizeof(double) * 10 * nn));
    SF_CUDA(cudaMalloc(&sp->samp, sizeof(double) * 8 * nn));
    SF_CUDA(cudaMemsetAsync(sp->gas, 0, sizeof(double) * 10 * nn, ctx->stream));
  }
  SF_CUDA(cudaMemsetAsync(sp->samp, 0, sizeof(double) * 8 * nn, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  sp->num_samples = 0;
  SF_API_END(ctx)
}

extern "C" int sf_samples_compute(sf_ctx* ctx, int32_t sid, double T_init, int64_t* num_samples) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(sp->samp, SF_ERR_STATE, "velocity sampling not set up (sf_samples_clear)");
  SF_CUDA(cudaSetDevice(ctx->device));
  const int nn = ctx->ni * ctx->nj;
  const double inv = sp->num_samples > 0 ? 1.0 / (double)sp->num_samples : 0.0;
  k_gas_fields<<<grid_for(nn, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(nn, sp->samp, inv, ctx->d_node_vol,
                                                                              sp->mass / KB, T_init, sp->gas);
  ctx->launches++;
  SF_CUDA(cudaGetLastError());
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  if (num_samples) *num_samples = sp->num_samples;
  SF_API_END(ctx)
}
