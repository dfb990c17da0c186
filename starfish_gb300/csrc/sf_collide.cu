// sf_collide.cu -- DSMC (Bird NTC) and MCC collisions on cell-sorted particles.
//
// DSMC.perform(mesh) (collisions/DSMC.java:194-256) bins particles by cell every call;
// here that binning is the species' counting sort, whose per-key offsets give each cell
// a contiguous run of particles.  collideCell (:259-350) then runs per cell with the
// reference's NTC count, remainder and (sigma g)max update; pair picks and acceptance use
// counter-based Philox streams keyed by (cell, step), so results match the reference in
// distribution (its global java.util.Random stream cannot be reproduced in parallel).
// Velocities are FP32 as stored; the selection count and cell state are FP64.
#include <climits>
#include <cmath>

#include "sf_internal.h"

using namespace sf;

namespace {

struct SigmaDev {
  int model;
  float c[4];
  float sigma0;    // BIRD463: pi d^2 for two equal diameters, 0.25 pi (d1+d2)^2
  float kT2_mr;    // BIRD463: 2 k T_ref / m_r
  float expo;      // omega - 1/2
  float inv_gamma; // 1 / Gamma(5/2 - omega) (Bird's gamma, Utils.gamma)
  float vss_inv;   // 0.5 (1/alpha1 + 1/alpha2)
  float c_bird;    // BIRD463 sigma g = c_bird (g^2)^expo_cr: sigma0 (2 k T_ref / m_r)^(omega - 1/2) / Gamma
  float expo_cr;   // 1/2 - (omega - 1/2)
};

// Sigma.eval (interactions/Sigma.java:121-195, SigmaPlus.java:54-76)
__device__ inline float sigma_eval(const SigmaDev& s, float g) {
  switch (s.model) {
    case SF_SIGMA_CONST: return s.c[0];
    case SF_SIGMA_INV: return g > 0.f ? s.c[0] / g : 0.f;
    case SF_SIGMA_POLY: {
      float v = s.c[0], gg = g;
      for (int i = 1; i < 4; i++) {
        v += s.c[i] * gg;
        gg *= gg;
      }
      return v;
    }
    case SF_SIGMA_LN: {
      if (!(g > 0.f)) return 0.f;
      const float v = s.c[0] + s.c[1] * logf(g);
      return v * v;
    }
    default:  // BIRD463
      if (!(g > 0.f)) return 0.f;
      return s.sigma0 * __powf(s.kT2_mr / (g * g), s.expo) * s.inv_gamma;
  }
}

// ModelElastic post-collision relative velocity (DSMC.java:389-427), equal masses
__device__ inline void elastic_vr(Philox& rng, float vss_inv, const float g[3], float g_mag, float vr[3]) {
  if (fabsf(vss_inv - 1.f) < 1e-4f) {
    const float B = 2.f * rng.uniformf() - 1.f;
    const float A = sqrtf(fmaxf(1.f - B * B, 0.f));
    vr[0] = B * g_mag;
    const float C = 2.f * (float)PI * rng.uniformf();
    float sC, cC;
    __sincosf(C, &sC, &cC);
    vr[1] = A * cC * g_mag;
    vr[2] = A * sC * g_mag;
  } else {
    const float B = 2.f * __powf(rng.uniformf(), vss_inv) - 1.f;
    const float A = sqrtf(fmaxf(1.f - B * B, 0.f));
    const float C = 2.f * (float)PI * rng.uniformf();
    float SC, OC;
    __sincosf(C, &SC, &OC);
    const float D = sqrtf(g[1] * g[1] + g[2] * g[2]);
    if (D > 1e-6f) {
      vr[0] = B * g[0] + A * SC * D;
      vr[1] = B * g[1] + A * (g_mag * g[2] * OC - g[0] * g[1] * SC) / D;
      vr[2] = B * g[2] - A * (g_mag * g[1] * OC + g[0] * g[2] * SC) / D;
    } else {
      vr[0] = B * g[1];
      vr[1] = A * OC * g[1];
      vr[2] = A * SC * g[1];
    }
  }
}

constexpr int DSMC_HEAVY_NSEL = 1024;    // candidate pairs beyond which a cell gets a CTA
// 1024 threads per dense cell: the rounds of a cell are sequential, so the densest cells'
// round count sets the kernel's length (0.206 -> 0.173 ms per jet step against 512, and
// 0.286 ms at 256)
constexpr int DSMC_HEAVY_THREADS = 1024;

// Everything a DSMC launch needs for one material pair (DSMC.java:259-350).  For a
// same-species pair P2/bins2 alias P1/bins1.
struct DsmcArgs {
  ParticlesView P1, P2;
  const int* bins1;  // per sort key: first slot of the cell's particles (+1: the next cell's)
  const int* bins2;
  int ntx, nkeys;
  const double* cell_vol;
  double2* state;    // per cell (sigma g)max, remainder
  double2* counts;   // per cell collision count, weight
  SigmaDev sg;
  double spwt1, spwt2;
  double dt;         // frequency * dt of the reference
  double nsel_den;   // Pab + (w2/w1) Pba (eq. 5 of Boyd's paper, DSMC.java:276-286)
  double real_w;     // 0.5 (w1 + w2): the weight summed per collision (DSMC.java:344)
  float rm1, rm2;    // m1/(m1+m2), m2/(m1+m2)
  float pab, pba;    // ModelElastic's variable-weight update probabilities (w2/w1, w1/w2)
  int boyd;          // the weights differ: Boyd's probabilistic velocity update
  uint64_t seed;
  uint32_t step;
  unsigned long long* n_coll;
  int* heavy;        // cells handed to k_dsmc_heavy (sort keys)
  unsigned* n_heavy;
  int heavy_cap;
  unsigned* work;    // k_dsmc_heavy's cell counter
  int* light;        // cells for k_dsmc (sort keys)
  unsigned* n_light;
  int* nsel;         // per cell: this call's candidate count (listed cells only)
};

// sigma(g) g of Sigma.eval (interactions/Sigma.java:121-195, SigmaPlus.java:54-76) from
// g^2.  Bird 4.63 is c g2^(1/2 - (omega - 1/2)) with c = sigma0 (2kT/m_r)^(omega - 1/2) /
// Gamma: one MUFU pair and no square root.
__device__ inline float sigma_cr_eval(const SigmaDev& s, float g2) {
  if (s.model == SF_SIGMA_BIRD463) return g2 > 0.f ? s.c_bird * __powf(g2, s.expo_cr) : 0.f;
  const float g = sqrtf(g2);
  return g * sigma_eval(s, g);
}

// One candidate pair (a of P1, b of P2) of collideCell: sigma g, the NTC acceptance
// sigma g / (sigma g)max, and ModelElastic.perform (DSMC.java:373-453) with the reduced
// masses and, for different weights, Boyd's update probabilities.  Returns whether the
// pair collided.
template <bool W>
__device__ inline bool collide_pair(const DsmcArgs& d, int64_t a, int64_t b, float smax, Philox& rng,
                                    float& smax_new, double& wsum) {
  const float2 va = d.P1.vxy[a], vb = d.P2.vxy[b];
  const float wa = d.P1.vz[a], wb = d.P2.vz[b];
  const float g[3] = {va.x - vb.x, va.y - vb.y, wa - wb};
  const float g2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  const float sigma_cr = sigma_cr_eval(d.sg, g2);
  smax_new = fmaxf(smax_new, sigma_cr);
  if (!(rng.uniformf() * smax < sigma_cr)) return false;  // sigma g / (sigma g)max > R
  const float g_mag = sqrtf(g2);
  const float vc[3] = {d.rm1 * va.x + d.rm2 * vb.x, d.rm1 * va.y + d.rm2 * vb.y, d.rm1 * wa + d.rm2 * wb};
  float vr[3];
  elastic_vr(rng, d.sg.vss_inv, g, g_mag, vr);
  bool boyd = d.boyd;
  float pab = d.pab, pba = d.pba;
  if (W) {
    // per-particle weights: Boyd's probabilities from the two particles' own weights, and
    // their mean in the collided-weight sum (DSMC.java:344, 431-452)
    const double w1 = d.spwt1 * (d.P1.w ? (double)d.P1.w[a] : 1.0);
    const double w2 = d.spwt2 * (d.P2.w ? (double)d.P2.w[b] : 1.0);
    boyd = w1 != w2;
    pab = (float)(w2 / w1);
    pba = (float)(w1 / w2);
    wsum += 0.5 * (w1 + w2);
  }
  const bool upd_a = !boyd || rng.uniformf() < pab;
  const bool upd_b = !boyd || rng.uniformf() < pba;
  if (upd_a) {
    d.P1.vxy[a] = make_float2(vc[0] + d.rm2 * vr[0], vc[1] + d.rm2 * vr[1]);
    d.P1.vz[a] = vc[2] + d.rm2 * vr[2];
  }
  if (upd_b) {
    d.P2.vxy[b] = make_float2(vc[0] - d.rm1 * vr[0], vc[1] - d.rm1 * vr[1]);
    d.P2.vz[b] = vc[2] - d.rm1 * vr[2];
  }
  return true;
}

__device__ inline bool is_prime(uint32_t x) {
  if (x < 4u) return x >= 2u;
  if ((x & 1u) == 0u) return false;
  for (uint32_t f = 3u; (uint64_t)f * f <= x; f += 2u)
    if (x % f == 0u) return false;
  return true;
}

// Smallest prime >= n (n >= 2), the 32 lanes of a warp testing consecutive candidates.
__device__ inline uint32_t warp_next_prime(uint32_t n) {
  const unsigned FULL = 0xffffffffu;
  for (uint32_t base = n;; base += 32u) {
    const unsigned b = __ballot_sync(FULL, is_prime(base + (threadIdx.x & 31u)));
    if (b) return base + (uint32_t)(__ffs(b) - 1);
  }
}

// uniform in [0, q) (bias below q / 2^64)
__device__ inline uint32_t rand_below(Philox& r, uint32_t q) {
  const uint64_t x = ((uint64_t)r.next_u32() << 32) | r.next_u32();
  return (uint32_t)__umul64hi(x, (uint64_t)q);
}

// Candidate pairs of a cell.  The reference draws each pair as p1 uniform and p2 != p1
// uniform, independently (DSMC.java:314-320; for two species p1 and p2 each uniform in
// their own list).  Here a round of pairs is collided in parallel, so its pairs must
// not share a particle.  A round maps the fixed inputs x = 0, 1, 2, ... through a random
// affine map s(x) = (a x + b) mod q of the prime field Z_q, q the smallest prime >= np,
// with a uniform in [1, q) and b uniform in [0, q): the maps of Z_q are sharply
// 2-transitive, so the images (s(x1), s(x2)) of two fixed distinct inputs are uniform
// over all ordered pairs of distinct elements.  Input pair k of a same-species round is
// (2k, 2k + 1); an image >= np is no particle and that candidate is not used (the
// others, conditioned on being particles, stay uniform over the cell's ordered pairs).
// Distinct inputs have distinct images, so the pairs of a round are disjoint.  For two
// species lane k takes s1(k) and s2(k) from two independent maps.  Rounds continue
// until nsel candidates have been used.
struct AffineMap {
  uint32_t q, a, b;
  __device__ inline uint32_t operator()(uint32_t x) const {
    if (q <= (1u << 22)) return (a * x + b) % q;  // a x + b < 2^32 for x < 1024
    return (uint32_t)(((uint64_t)a * x + b) % q);
  }
  __device__ inline uint32_t next(uint32_t y) const {  // s(x + 1) from y = s(x)
    const uint32_t z = y + a;
    return z >= q ? z - q : z;
  }
  __device__ inline void draw(Philox& r) {
    a = 1u + rand_below(r, q - 1u);
    b = rand_below(r, q);
  }
};

// Bound on the rounds of a cell: every round uses each considered candidate with
// probability > 1/4, so this is never reached in practice; it only bounds the loop.
__device__ inline int max_rounds(int nsel) { return nsel > (1 << 26) ? INT_MAX : 64 + 16 * nsel; }

// NTC selection count of collideCell (DSMC.java:272-304): nsel and the new remainder;
// false when the cell has too few particles (the reference returns before updating rem)
template <bool PAIR>
__device__ inline bool cell_nsel(const DsmcArgs& d, int np1, int np2, int c, double2 st, int& nsel, double& rem) {
  if (PAIR ? (np1 < 1 || np2 < 1) : (np1 < 2)) return false;
  double nsel_f = (((double)np1 * d.spwt1 / d.cell_vol[c]) * (double)np2 * d.dt * st.x) / d.nsel_den;
  if (PAIR) nsel_f *= 2.0;  // "q-p" collisions are not done separately from "p-q"
  nsel_f += st.y;
  nsel = (int)nsel_f;
  rem = nsel_f - nsel;
  if ((double)nsel > (double)np1 * (double)np2) {
    nsel = (int)((double)np1 * (double)np2);
    rem = 0.0;
  }
  return true;
}

// The NTC plan of every cell, one thread per cell: the selection count nsel and the new
// remainder of collideCell (DSMC.java:272-304; the remainder is stored here), and the
// cell's place in the list of k_dsmc (a warp per cell) or, beyond DSMC_HEAVY_NSEL
// candidates with at least 128 particles on each side, of k_dsmc_heavy (a CTA per cell).
// Cells with fewer particles than a pair, or no candidate this call, are in neither.  The
// FP64 arithmetic of nsel runs once per cell instead of on every lane of a warp.
template <bool PAIR>
__global__ void k_dsmc_plan(MeshView m, DsmcArgs d) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int ncx = m.ni - 1, nc = ncx * (m.nj - 1);
  const int stride = (int)(gridDim.x * blockDim.x);
  for (int c0 = (int)(blockIdx.x * blockDim.x); c0 < nc; c0 += stride) {
    const int c = c0 + (int)threadIdx.x;
    int list = 0;  // 1 light, 2 heavy
    int key = 0;
    if (c < nc) {
      const int j = c / ncx, i = c - j * ncx;
      key = (int)cell_key(i, j, d.ntx);
      const int s1 = d.bins1[key], np1 = d.bins1[key + 1] - s1;
      const int np2 = PAIR ? d.bins2[key + 1] - d.bins2[key] : np1;
      double2* stp = &d.state[c];
      int nsel;
      double rem;
      if (cell_nsel<PAIR>(d, np1, np2, c, *stp, nsel, rem)) {
        stp->y = rem;
        if (nsel > 0) {
          d.nsel[c] = nsel;
          list = (nsel > DSMC_HEAVY_NSEL && min(np1, np2) >= 128) ? 2 : 1;
        }
      }
    }
    // warp-aggregated appends to the two lists
#pragma unroll
    for (int l = 1; l <= 2; l++) {
      const unsigned mk = __ballot_sync(FULL, list == l);
      if (!mk) continue;
      const int leader = __ffs(mk) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(l == 1 ? d.n_light : d.n_heavy, (unsigned)__popc(mk));
      base = __shfl_sync(FULL, base, leader);
      if (list == l) (l == 1 ? d.light : d.heavy)[base + __popc(mk & ((1u << lane) - 1u))] = key;
    }
  }
}

// DSMC.collideCell for the cells of k_dsmc_plan's light list, one warp per cell, warps
// striding over the list.  The acceptance and the (sigma g)max update are the
// reference's; candidates come in rounds of up to 32 disjoint pairs (AffineMap), one per
// lane.
// W: a species holds per-particle weights
template <bool PAIR, bool W>
__global__ void __launch_bounds__(128) k_dsmc(MeshView m, DsmcArgs d) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warps = (int)(gridDim.x * blockDim.x) >> 5;
  const int nl = (int)*d.n_light;
  for (int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); e < nl; e += warps) {
    const int key = d.light[e];
    int i, j;
    key_cell((uint32_t)key, d.ntx, i, j);
    const int c = j * (m.ni - 1) + i;
    const int s1 = d.bins1[key], np1 = d.bins1[key + 1] - s1;
    const int s2 = PAIR ? d.bins2[key] : s1;
    const int np2 = PAIR ? d.bins2[key + 1] - s2 : np1;
    const int nsel = d.nsel[c];
    const double smax_old = d.state[c].x;  // (sigma g)max
    Philox rng(d.seed, RNG_DSMC, (uint64_t)c * 32u + (uint64_t)lane, d.step);
    AffineMap s1m, s2m;
    s1m.q = warp_next_prime((uint32_t)np1);
    s2m.q = PAIR ? warp_next_prime((uint32_t)np2) : s1m.q;
    float smax_new = 0.f;
    const float smax = (float)smax_old;
    int ncol = 0;
    double wsum = 0.0;  // collided weight (per-particle weights)
    const int per_round = PAIR ? min(32, min(np1, np2)) : min(32, np1 / 2);
    int left = nsel;
    for (int round = 0, cap = max_rounds(nsel); left > 0 && round < cap; round++) {
      const int mr = min(per_round, left);
      if (lane == 0) {
        s1m.draw(rng);
        if (PAIR) s2m.draw(rng);
      }
      s1m.a = __shfl_sync(FULL, s1m.a, 0);
      s1m.b = __shfl_sync(FULL, s1m.b, 0);
      if (PAIR) {
        s2m.a = __shfl_sync(FULL, s2m.a, 0);
        s2m.b = __shfl_sync(FULL, s2m.b, 0);
      }
      bool used = false;
      if (lane < mr) {
        uint32_t p1, p2;
        if (PAIR) {
          p1 = s1m((uint32_t)lane);
          p2 = s2m((uint32_t)lane);
        } else {
          p1 = s1m(2u * lane);
          p2 = s1m.next(p1);
        }
        used = p1 < (uint32_t)np1 && p2 < (uint32_t)np2;
        if (used && collide_pair<W>(d, s1 + (int64_t)p1, s2 + (int64_t)p2, smax, rng, smax_new, wsum)) ncol++;
      }
      left -= __popc(__ballot_sync(FULL, used));
      __syncwarp();  // this round's velocities are visible to the next round's lanes
    }
    for (int o = 16; o > 0; o >>= 1) {
      smax_new = fmaxf(smax_new, __shfl_xor_sync(FULL, smax_new, o));
      ncol += __shfl_xor_sync(FULL, ncol, o);
      if (W) wsum += __shfl_xor_sync(FULL, wsum, o);
    }
    if (lane == 0) {
      if (smax_new > 0.f) d.state[c].x = (double)smax_new;
      if (ncol) {
        double2 cs = d.counts[c];
        cs.x += ncol;
        cs.y += W ? wsum : ncol * d.real_w;
        d.counts[c] = cs;
        atomicAdd(d.n_coll, (unsigned long long)ncol);
      }
    }
  }
}

// The cells handed over by k_dsmc, one CTA of DSMC_HEAVY_THREADS per cell: rounds of up
// to DSMC_HEAVY_THREADS disjoint pairs (the same AffineMap selection), the CTA
// synchronising between rounds.
template <bool PAIR, bool W>
__global__ void __launch_bounds__(DSMC_HEAVY_THREADS) k_dsmc_heavy(MeshView m, DsmcArgs d) {
  __shared__ int s_idx;
  __shared__ uint32_t s_q[2], s_ab[2][4];  // the maps of this round and the next
  __shared__ float s_max[DSMC_HEAVY_THREADS / 32];
  __shared__ int s_n[DSMC_HEAVY_THREADS / 32];
  __shared__ double s_ws[DSMC_HEAVY_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nh = min((int)*d.n_heavy, d.heavy_cap);
  for (;;) {
    if (tid == 0) s_idx = (int)atomicAdd(d.work, 1u);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= nh) break;
    const int key = d.heavy[idx];
    int i, j;
    key_cell((uint32_t)key, d.ntx, i, j);
    const int c = j * (m.ni - 1) + i;
    const int s1 = d.bins1[key], np1 = d.bins1[key + 1] - s1;
    const int s2 = PAIR ? d.bins2[key] : s1;
    const int np2 = PAIR ? d.bins2[key + 1] - s2 : np1;
    const int nsel = d.nsel[c];
    const double smax_old = d.state[c].x;
    if (wid == 0) {
      const uint32_t q1 = warp_next_prime((uint32_t)np1);
      const uint32_t q2 = PAIR ? warp_next_prime((uint32_t)np2) : q1;
      if (lane == 0) {
        s_q[0] = q1;
        s_q[1] = q2;
      }
    }
    __syncthreads();
    AffineMap s1m, s2m;
    s1m.q = s_q[0];
    s2m.q = s_q[1];
    Philox rng(d.seed, RNG_DSMC_HEAVY, (uint64_t)c * DSMC_HEAVY_THREADS + (uint64_t)tid, d.step);
    float smax_new = 0.f;
    const float smax = (float)smax_old;
    int ncol = 0;
    double wsum = 0.0;
    const int per_round = PAIR ? min(DSMC_HEAVY_THREADS, min(np1, np2)) : min(DSMC_HEAVY_THREADS, np1 / 2);
    int left = nsel;
    // thread 0 draws the maps one round ahead, so that a round waits at one barrier only
    auto draw = [&](uint32_t* ab) {  // into copies: thread 0 still uses this round's maps
      AffineMap t1 = s1m, t2 = s2m;
      t1.draw(rng);
      ab[0] = t1.a;
      ab[1] = t1.b;
      if (PAIR) {
        t2.draw(rng);
        ab[2] = t2.a;
        ab[3] = t2.b;
      }
    };
    if (tid == 0) draw(s_ab[0]);
    __syncthreads();
    for (int round = 0, cap = max_rounds(nsel); left > 0 && round < cap; round++) {
      const int mr = min(per_round, left);
      const uint32_t* ab = s_ab[round & 1];
      s1m.a = ab[0];
      s1m.b = ab[1];
      if (PAIR) {
        s2m.a = ab[2];
        s2m.b = ab[3];
      }
      if (tid == 0) draw(s_ab[(round + 1) & 1]);  // read by the next round, after the barrier below
      bool used = false;
      if (tid < mr) {
        uint32_t p1, p2;
        if (PAIR) {
          p1 = s1m((uint32_t)tid);
          p2 = s2m((uint32_t)tid);
        } else {
          p1 = s1m(2u * tid);
          p2 = s1m.next(p1);
        }
        used = p1 < (uint32_t)np1 && p2 < (uint32_t)np2;
        if (used && collide_pair<W>(d, s1 + (int64_t)p1, s2 + (int64_t)p2, smax, rng, smax_new, wsum)) ncol++;
      }
      // the count of used candidates; also orders this round's velocities and the next
      // round's maps before the next round
      left -= __syncthreads_count(used);
    }
    for (int o = 16; o > 0; o >>= 1) {
      smax_new = fmaxf(smax_new, __shfl_xor_sync(0xffffffffu, smax_new, o));
      ncol += __shfl_xor_sync(0xffffffffu, ncol, o);
      if (W) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
    }
    if (lane == 0) {
      s_max[wid] = smax_new;
      s_n[wid] = ncol;
      if (W) s_ws[wid] = wsum;
    }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < DSMC_HEAVY_THREADS / 32; w++) {
        smax_new = fmaxf(smax_new, s_max[w]);
        ncol += s_n[w];
        if (W) wsum += s_ws[w];
      }
      if (smax_new > 0.f) d.state[c].x = (double)smax_new;
      if (ncol) {
        double2 cs = d.counts[c];
        cs.x += ncol;
        cs.y += W ? wsum : ncol * d.real_w;
        d.counts[c] = cs;
        atomicAdd(d.n_coll, (unsigned long long)ncol);
      }
    }
    __syncthreads();  // s_max / s_n are reused by the next cell
  }
}

struct TargetView {
  const float* den;
  const float* u;
  const float* v;
  const float* w;
  const float* T;
  float mass;
};

__device__ inline float gather_node(const float* f, int ni, int i, int j, float fx, float fy) {
  const int u = j * ni + i;
  return (1.f - fx) * (1.f - fy) * f[u] + fx * (1.f - fy) * f[u + 1] + fx * fy * f[u + ni + 1] +
         (1.f - fx) * fy * f[u + ni];
}

// Per-collision sums of MCC.perform (MCC.java:198-219) and the products of
// ModelIonization (:304-356).  Every pointer may be null (not accumulated).
struct MccExtra {
  double* S;          // ni*nj: target energy term mpw (E1 - E2) / (dt V), Field2D.scatter
  double* count_sum;  // ni*nj at node (int) lc: collisions
  double* real_sum;   // ni*nj at node (int) lc: collided weight
  double* dn;         // ni*nj at node (int) lc: product weight created (target delta-N)
  double spwt;        // source weight (uniform)
  double dt;
  // ionization (model SF_MCC_IONIZATION)
  double e_ion;       // eV
  double prod_mass, prod_spwt, spwt_ratio;  // spwt_ratio = source spwt / product spwt
  float qm_halfdt_src, qm_halfdt_prod;      // (q/m) dt/2 of the addParticle rewind
  ParticlesView Pe;   // source species: new electrons from slot Pe.n
  ParticlesView Pi;   // product species: new ions from slot Pi.n
  int64_t cap_e, cap_i;
};

// Mesh.nodeVol at a fractional position (Mesh.java:961-1020) on a single mesh: the
// control volume [i0 -/+ 1/2] x [j0 -/+ 1/2] clipped to the mesh (Mesh.controlVolumeLCs;
// the corner moves next to INSULATOR nodes do not apply on MCC meshes without them).
__device__ double node_vol_at(const MeshView& m, double i0, double j0) {
  const double wi = fmin(i0 + 0.5, (double)(m.ni - 1)) - fmax(i0 - 0.5, 0.0);
  const double wj = fmin(j0 + 0.5, (double)(m.nj - 1)) - fmax(j0 - 0.5, 0.0);
  const double area = wi * m.dh[0] * wj * m.dh[1];
  if (m.domain == SF_DOMAIN_XY) return area;
  double r;
  if (m.domain == SF_DOMAIN_RZ) {
    double ir = i0;
    if (i0 == 0.0) ir = 0.25;
    else if (i0 == m.ni - 1) ir = i0 - 0.25;
    r = m.x0[0] + ir * m.dh[0];
  } else {
    double jr = j0;
    if (j0 == 0.0) jr = 0.25;
    else if (j0 == m.nj - 1) jr = j0 - 0.25;
    r = m.x0[1] + jr * m.dh[1];
  }
  return 2.0 * PI * area * r;
}

// Field2D.scatter (Field2D.java:244-295) with the Ruyten RZ / ZR weights, FP64 atomics
__device__ void scatter_fp64(const MeshView& m, double* f, double fi, double fj, double val) {
  const int i = (int)fi, j = (int)fj;
  if (i < 0 || j < 0 || i >= m.ni - 1 || j >= m.nj - 1) return;
  double di = fi - i, dj = fj - j;
  if (m.domain == SF_DOMAIN_RZ) {
    const double rp = m.x0[0] + (i + 1) * m.dh[0], rm = m.x0[0] + i * m.dh[0], r = m.x0[0] + fi * m.dh[0];
    di = 1 - (0.5 * (rp - r) * (2 * rp + 3 * rm - r) / (rp * rp - rm * rm));
  } else if (m.domain == SF_DOMAIN_ZR) {
    const double rp = m.x0[1] + (j + 1) * m.dh[1], rm = m.x0[1] + j * m.dh[1], r = m.x0[1] + fj * m.dh[1];
    dj = 1 - (0.5 * (rp - r) * (2 * rp + 3 * rm - r) / (rp * rp - rm * rm));
  }
  const int u = j * m.ni + i;
  atomicAdd(&f[u], (1 - di) * (1 - dj) * val);
  atomicAdd(&f[u + 1], di * (1 - dj) * val);
  atomicAdd(&f[u + m.ni + 1], di * dj * val);
  atomicAdd(&f[u + m.ni], (1 - di) * dj * val);
}

// Utils.isotropicVel (core/common/Utils.java:121-136)
__device__ inline void isotropic_vel(Philox& r, double mag, double v[3]) {
  const double theta = 2 * PI * r.uniform();
  const double R = -1.0 + 2 * r.uniform();
  const double a = sqrt(fmax(1 - R * R, 0.0));
  const double am = fabs(mag);
  v[0] = cos(theta) * a * am;
  v[1] = sin(theta) * a * am;
  v[2] = R * am;
}

// KineticMaterial.addParticle (KineticMaterial.java:776-796): the new particle at the
// source particle's place with the -dt/2 velocity rewind; false past the capacity
__device__ bool mcc_append(const MeshView& m, const ParticlesView& Q, int64_t cap, unsigned long long* ctr, uint32_t cell,
                           float2 f, const double v[3], float qm_halfdt, float wnew = 1.f) {
  const int64_t d = Q.n + (int64_t)atomicAdd(ctr, 1ULL);
  if (d >= cap) return false;
  const float2 e = gather_efield(m.E, m.ni, cell_i(cell), cell_j(cell), f.x, f.y);
  Q.cell[d] = cell;
  Q.frac[d] = f;
  Q.vxy[d] = make_float2((float)v[0] - qm_halfdt * e.x, (float)v[1] - qm_halfdt * e.y);
  Q.vz[d] = (float)v[2];
  if (Q.w) Q.w[d] = wnew;  // fraction of the species weight
  return true;
}

// MCC.perform(mesh) per particle (collisions/MCC.java:167-221)
__global__ void k_mcc(MeshView m, ParticlesView P, TargetView tg, SigmaDev sg, int model, float src_mass, float dt,
                      uint64_t seed, uint32_t step, unsigned long long* __restrict__ cnt, MccExtra ex) {
  const float KBf = 1.3806503e-23f;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = P.cell[p];
    if (c == DEAD) continue;
    const int i = cell_i(c), j = cell_j(c);
    const float2 f = P.frac[p];
    const float den = gather_node(tg.den, m.ni, i, j, f.x, f.y);
    if (den <= 0.f) continue;
    const float tu = tg.u ? gather_node(tg.u, m.ni, i, j, f.x, f.y) : 0.f;
    const float tv = tg.v ? gather_node(tg.v, m.ni, i, j, f.x, f.y) : 0.f;
    const float tw = tg.w ? gather_node(tg.w, m.ni, i, j, f.x, f.y) : 0.f;
    float2 vxy = P.vxy[p];
    float vz = P.vz[p];
    const float gx = tu - vxy.x, gy = tv - vxy.y, gz = tw - vz;
    const float g = sqrtf(gx * gx + gy * gy + gz * gz);
    const float Pc = 1.f - __expf(-sigma_eval(sg, g) * g * dt * den);
    Philox rng(seed, RNG_MCC, (uint64_t)p, step);
    if (Pc < rng.uniformf()) continue;
    const float wp = P.w ? P.w[p] : 1.f;  // the particle's fraction of the species weight
    // Material.sampleMaxwellianVelocity (Material.java:880-896): mean + SampleMaxw3D(v_th)
    float T = gather_node(tg.T, m.ni, i, j, f.x, f.y);
    if (T < 0.f) T = 0.f;
    const float vth = sqrtf(2.f * KBf * T / tg.mass);
    float vt[3] = {tu, tv, tw};
    for (int d = 0; d < 3; d++) {
      float s = 0.f;
      for (int k = 0; k < 12; k++) s += rng.uniformf();
      vt[d] += (vth * 1.2f) * 0.70710678f * (s - 6.f);
    }
    // pre-collision "energy" 0.5 m |v| (Vec.mag3, as in MCC.java:204)
    const double E1 = 0.5 * (double)src_mass * sqrt((double)vxy.x * vxy.x + (double)vxy.y * vxy.y + (double)vz * vz);
    if (model == SF_MCC_IONIZATION) {
      // ModelIonization (MCC.java:304-356): the source electron keeps a random share of
      // the energy left after ionization; a second electron (with the same speed, as in
      // the reference) and (int)(spwt_src / spwt_prod + rnd) product ions at the neutral
      // temperature are added where the collision happened
      const double e1 = 0.5 * (double)src_mass * ((double)vxy.x * vxy.x + (double)vxy.y * vxy.y + (double)vz * vz) / QE;
      const double e2 = e1 - ex.e_ion;
      if (e2 >= 0) {
        const double e2a = rng.uniform() * e2;
        const double speed2a = sqrt(e2a * QE * 2 / (double)src_mass);
        double vs[3], v2b[3];
        isotropic_vel(rng, speed2a, vs);
        vxy = make_float2((float)vs[0], (float)vs[1]);
        vz = (float)vs[2];
        double Tt = (double)gather_node(tg.T, m.ni, i, j, f.x, f.y);
        if (Tt <= 0) Tt = 100;
        isotropic_vel(rng, speed2a, v2b);
        // the second electron carries the source electron's weight (MCC.java:335)
        if (!mcc_append(m, ex.Pe, ex.cap_e, &cnt[1], c, f, v2b, ex.qm_halfdt_src, wp)) atomicAdd(&cnt[3], 1ULL);
        const int mp_gen = (int)(ex.spwt_ratio * (double)wp + rng.uniform());
        if (mp_gen > 0) {
          const double v_th = sqrt(2 * KB * Tt / ex.prod_mass);
          for (int k = 0; k < mp_gen; k++) {
            double v3[3];
            for (int d = 0; d < 3; d++) v3[d] = (v_th * 1.2) * rng.maxw1d_unit();  // Utils.SampleMaxw3D
            if (!mcc_append(m, ex.Pi, ex.cap_i, &cnt[2], c, f, v3, ex.qm_halfdt_prod)) atomicAdd(&cnt[3], 1ULL);
          }
          if (ex.dn) {
            const int ii = i + (f.x >= 1.f), jj = j + (f.y >= 1.f);
            atomicAdd(&ex.dn[jj * m.ni + ii], ex.prod_spwt * mp_gen);
          }
        }
      }
    } else if (model == SF_MCC_CEX) {
      vxy = make_float2(vt[0], vt[1]);
      vz = vt[2];
    } else {
      // ModelMEX (MCC.java:242-285): isotropic scattering in the centre-of-mass frame
      const float rm1 = src_mass / (src_mass + tg.mass), rm2 = tg.mass / (src_mass + tg.mass);
      const float gg[3] = {vxy.x - vt[0], vxy.y - vt[1], vz - vt[2]};
      const float g_mag = sqrtf(gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2]);
      const float vc[3] = {rm1 * vxy.x + rm2 * vt[0], rm1 * vxy.y + rm2 * vt[1], rm1 * vz + rm2 * vt[2]};
      const float B = 2.f * rng.uniformf() - 1.f;
      const float A = sqrtf(fmaxf(1.f - B * B, 0.f));
      const float C = 2.f * (float)PI * rng.uniformf();
      float sC, cC;
      __sincosf(C, &sC, &cC);
      const float vr[3] = {B * g_mag, A * cC * g_mag, A * sC * g_mag};
      vxy = make_float2(vc[0] + vr[0] * rm2, vc[1] + vr[1] * rm2);
      vz = vc[2] + vr[2] * rm2;
    }
    P.vxy[p] = vxy;
    P.vz[p] = vz;
    atomicAdd(&cnt[0], 1ULL);
    const double li = i + (double)f.x, lj = j + (double)f.y;
    if (ex.S) {
      const double E2 = 0.5 * (double)src_mass * sqrt((double)vxy.x * vxy.x + (double)vxy.y * vxy.y + (double)vz * vz);
      scatter_fp64(m, ex.S, li, lj, ex.spwt * (double)wp * (E1 - E2) / (ex.dt * node_vol_at(m, li, lj)));
    }
    if (ex.count_sum) {
      const int u = (j + (f.y >= 1.f)) * m.ni + i + (f.x >= 1.f);
      atomicAdd(&ex.count_sum[u], 1.0);
      atomicAdd(&ex.real_sum[u], ex.spwt * (double)wp);
    }
  }
}

// Utils.gamma, Bird's approximation (core/common/Utils.java:218-236)
double bird_gamma(double X) {
  double A = 1., Y = X;
  if (Y < 1.0) {
    A = A / Y;
  } else {
    do {
      Y = Y - 1;
      if (Y >= 1.) A = A * Y;
    } while (Y >= 1.);
  }
  return A * (1. - 0.5748646 * Y + 0.9512363 * Y * Y - 0.6998588 * Y * Y * Y + 0.4245549 * Y * Y * Y * Y -
              0.1010678 * Y * Y * Y * Y * Y);
}

// Sigma.init for the pair (mat1, mat2) (SigmaPlus.java:54-66 for Bird 4.63) and the pair's
// vss_inv (DSMC.java:81).  s2 carries the second material's diameter, reference
// temperature, viscosity index and VSS alpha; null for a same-material pair.
SigmaDev make_sigma(const sf_sigma* s, const sf_sigma* s2, double m1, double m2) {
  SF_REQUIRE(s, SF_ERR_ARG, "null sigma");
  SF_REQUIRE(s->model >= SF_SIGMA_CONST && s->model <= SF_SIGMA_BIRD463, SF_ERR_ARG, "bad sigma model");
  if (!s2) s2 = s;
  SigmaDev d{};
  d.model = s->model;
  for (int k = 0; k < 4; k++) d.c[k] = (float)s->c[k];
  if (s->model == SF_SIGMA_BIRD463) {
    SF_REQUIRE(s->diam > 0 && s->T_ref > 0 && s2->diam > 0 && s2->T_ref > 0, SF_ERR_ARG,
               "Bird 4.63 needs diam and T_ref");
    const double d_ref = s->diam + s2->diam;
    const double T_ref = 0.5 * (s->T_ref + s2->T_ref);
    const double omega = 0.5 * (s->omega + s2->omega);
    const double mr = m1 * m2 / (m1 + m2);
    const double sigma0 = 0.25 * PI * d_ref * d_ref;
    const double kT2_mr = 2.0 * KB * T_ref / mr;
    const double inv_gamma = 1.0 / bird_gamma(2.5 - omega);
    d.sigma0 = (float)sigma0;
    d.kT2_mr = (float)kT2_mr;
    d.expo = (float)(omega - 0.5);
    d.inv_gamma = (float)inv_gamma;
    d.c_bird = (float)(sigma0 * std::pow(kT2_mr, omega - 0.5) * inv_gamma);
    d.expo_cr = (float)(0.5 - (omega - 0.5));
  }
  const double a1 = s->vss_alpha > 0 ? s->vss_alpha : 1.0;
  const double a2 = s2->vss_alpha > 0 ? s2->vss_alpha : 1.0;
  d.vss_inv = (float)(0.5 * (1.0 / a1 + 1.0 / a2));
  return d;
}

}  // namespace

struct SfDsmcState {
  int sid1 = -1, sid2 = -1;
  double2* state = nullptr;   // per cell (sigma g)max, remainder
  double2* counts = nullptr;  // per cell collision count, weight
  double* cell_vol = nullptr;
  int* bins1 = nullptr;       // two species: the first one's sort bins (the second uses ctx->bins)
  int* nsel = nullptr;        // per cell: candidate count of the current call (k_dsmc_plan)
  int* light = nullptr;       // cells of k_dsmc (sort keys), up to one per cell
};

// per-context DSMC state of a material pair; freed with the context through the destroy hook
static SfDsmcState* find_dsmc(sf_ctx* ctx, int sid1, int sid2) {
  for (SfDsmcState* st : ctx->dsmc)
    if (st->sid1 == sid1 && st->sid2 == sid2) return st;
  return nullptr;
}

static SfDsmcState* dsmc_state(sf_ctx* ctx, int sid1, int sid2, double sig_cr_max0) {
  if (SfDsmcState* st = find_dsmc(ctx, sid1, sid2)) return st;
  SfDsmcState* st = new SfDsmcState();
  ctx->dsmc.push_back(st);
  st->sid1 = sid1;
  st->sid2 = sid2;
  const int nc = ctx->ncells();
  SF_CUDA(cudaMalloc(&st->state, sizeof(double2) * nc));
  SF_CUDA(cudaMalloc(&st->counts, sizeof(double2) * nc));
  SF_CUDA(cudaMalloc(&st->cell_vol, sizeof(double) * nc));
  SF_CUDA(cudaMalloc(&st->nsel, sizeof(int) * nc));
  SF_CUDA(cudaMalloc(&st->light, sizeof(int) * nc));
  if (sid1 != sid2) SF_CUDA(cudaMalloc(&st->bins1, sizeof(int) * ((size_t)ctx->nkeys + 1)));
  std::vector<double2> s0(nc, make_double2(sig_cr_max0, 0.0));
  copy_wait(st->state, s0.data(), sizeof(double2) * nc, cudaMemcpyHostToDevice, ctx->stream);
  zero_wait(st->counts, sizeof(double2) * nc, ctx->stream);
  // Mesh.cellVol = nodeVol(i + 1/2, j + 1/2) (core/domain/Mesh.java:1038-1040)
  std::vector<double> cv(nc);
  for (int j = 0; j < ctx->nj - 1; j++)
    for (int i = 0; i < ctx->ni - 1; i++) {
      const double area = ctx->dh[0] * ctx->dh[1];
      double v = area;
      if (ctx->domain == SF_DOMAIN_RZ) v = 2 * PI * area * (ctx->x0[0] + (i + 0.5) * ctx->dh[0]);
      if (ctx->domain == SF_DOMAIN_ZR) v = 2 * PI * area * (ctx->x0[1] + (j + 0.5) * ctx->dh[1]);
      cv[(size_t)j * (ctx->ni - 1) + i] = v;
    }
  copy_wait(st->cell_vol, cv.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, ctx->stream);
  return st;
}

void sf_collide_destroy_internal(sf_ctx* ctx) {
  for (SfDsmcState* st : ctx->dsmc) {
    cudaFree(st->state);
    cudaFree(st->counts);
    cudaFree(st->cell_vol);
    cudaFree(st->bins1);
    cudaFree(st->nsel);
    cudaFree(st->light);
    delete st;
  }
  ctx->dsmc.clear();
  if (ctx->mcc_target) {
    cudaFree(ctx->mcc_target);
    ctx->mcc_target = nullptr;
  }
  if (ctx->mcc_sums) {
    cudaFree(ctx->mcc_sums);
    ctx->mcc_sums = nullptr;
  }
  if (ctx->mcc_cnt) {
    cudaFree(ctx->mcc_cnt);
    ctx->mcc_cnt = nullptr;
  }
}

namespace {

// DSMC.perform(mesh) for the pair (sid1, sid2): cell binning by the species' counting
// sorts, then collideCell per cell (k_dsmc, k_dsmc_heavy).
void dsmc_run(sf_ctx* ctx, int sid1, int sid2, const sf_sigma* sigma, const sf_sigma* sigma2, double dt,
              double sig_cr_max0, int64_t* n_coll) {
  // the binning sort drops removed slots itself: the removals of pushes and sources that
  // did not wait need not be read first
  SfSpecies* sp1 = get_species_nowait(ctx, sid1);
  SfSpecies* sp2 = get_species_nowait(ctx, sid2);
  SF_REQUIRE(dt > 0 && sig_cr_max0 > 0, SF_ERR_ARG, "dt and sig_cr_max must be positive");
  SF_CUDA(cudaSetDevice(ctx->device));
  const bool pair = sid1 != sid2;
  SfDsmcState* st = dsmc_state(ctx, sid1, sid2, sig_cr_max0);
  DsmcArgs d{};
  d.sg = make_sigma(sigma, pair ? sigma2 : nullptr, sp1->mass, sp2->mass);
  // DSMC.perform(mesh) bins particles by cell on every call: the counting sort.  With two
  // species the first one's bins are kept aside before the second sort reuses ctx->bins.
  launch_sort(ctx, sp1);
  if (pair) {
    SF_CUDA(cudaMemcpyAsync(st->bins1, ctx->bins, sizeof(int) * ((size_t)ctx->nkeys + 1), cudaMemcpyDeviceToDevice,
                            ctx->stream));
    launch_sort(ctx, sp2);
  }
  d.P1 = sp1->cur;
  d.P2 = sp2->cur;
  d.bins1 = pair ? st->bins1 : ctx->bins;
  d.bins2 = ctx->bins;
  d.ntx = ctx->ntx;
  d.nkeys = ctx->nkeys;
  d.cell_vol = st->cell_vol;
  d.state = st->state;
  d.counts = st->counts;
  d.spwt1 = sp1->spwt;
  d.spwt2 = sp2->spwt;
  d.dt = dt;
  // eq. 5 of Boyd's paper (DSMC.java:276-286)
  const double Pab = std::min(1.0, sp2->spwt / sp1->spwt), Pba = std::min(1.0, sp1->spwt / sp2->spwt);
  d.nsel_den = Pab + (sp2->spwt / sp1->spwt) * Pba;
  d.real_w = 0.5 * (sp1->spwt + sp2->spwt);
  d.rm1 = (float)(sp1->mass / (sp1->mass + sp2->mass));
  d.rm2 = (float)(sp2->mass / (sp1->mass + sp2->mass));
  d.boyd = sp1->spwt != sp2->spwt;
  d.pab = (float)(sp2->spwt / sp1->spwt);
  d.pba = (float)(sp1->spwt / sp2->spwt);
  d.seed = ctx->seed ^ 0xD5C0ULL;
  d.step = ctx->rng_epoch++;
  // counters[6]: collisions; as unsigned: [3] the number of heavy cells, [4] the
  // heavy-cell work counter, [5] the number of light cells.  The heavy-cell list lives in
  // bins_tmp (the sort's write cursors, free once the particles are binned).
  SF_CUDA(cudaMemsetAsync(ctx->counters + 3, 0, 4 * sizeof(unsigned long long), ctx->stream));
  d.n_coll = ctx->counters + 6;
  d.heavy = ctx->bins_tmp;
  d.n_heavy = reinterpret_cast<unsigned*>(ctx->counters + 3);
  d.heavy_cap = ctx->nkeys;
  d.work = reinterpret_cast<unsigned*>(ctx->counters + 4);
  d.light = st->light;
  d.n_light = reinterpret_cast<unsigned*>(ctx->counters + 5);
  d.nsel = st->nsel;
  {
    TimedScope ts(ctx, "dsmc");
    const bool wt = sp1->weighted || sp2->weighted;
    const int pgrid = grid_for((int64_t)ctx->ncells(), 256, ctx->num_sms * 8);
    if (pair)
      k_dsmc_plan<true><<<pgrid, 256, 0, ctx->stream>>>(ctx->mesh_view(), d);
    else
      k_dsmc_plan<false><<<pgrid, 256, 0, ctx->stream>>>(ctx->mesh_view(), d);
    if (pair && wt) {
      k_dsmc<true, true><<<ctx->num_sms * 16, 128, 0, ctx->stream>>>(ctx->mesh_view(), d);
      k_dsmc_heavy<true, true><<<ctx->num_sms, DSMC_HEAVY_THREADS, 0, ctx->stream>>>(ctx->mesh_view(), d);
    } else if (pair) {
      k_dsmc<true, false><<<ctx->num_sms * 16, 128, 0, ctx->stream>>>(ctx->mesh_view(), d);
      k_dsmc_heavy<true, false><<<ctx->num_sms, DSMC_HEAVY_THREADS, 0, ctx->stream>>>(ctx->mesh_view(), d);
    } else if (wt) {
      k_dsmc<false, true><<<ctx->num_sms * 16, 128, 0, ctx->stream>>>(ctx->mesh_view(), d);
      k_dsmc_heavy<false, true><<<ctx->num_sms, DSMC_HEAVY_THREADS, 0, ctx->stream>>>(ctx->mesh_view(), d);
    } else {
      k_dsmc<false, false><<<ctx->num_sms * 16, 128, 0, ctx->stream>>>(ctx->mesh_view(), d);
      k_dsmc_heavy<false, false><<<ctx->num_sms, DSMC_HEAVY_THREADS, 0, ctx->stream>>>(ctx->mesh_view(), d);
    }
    ctx->launches += 3;
  }
  SF_CUDA(cudaGetLastError());
  unsigned long long nc = 0;
  if (!n_coll) return;  // nothing to read: the collisions stay queued on the context's stream
  SF_CUDA(cudaMemcpyAsync(&nc, ctx->counters + 6, sizeof(nc), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  timer_collect(ctx);
  *n_coll = (int64_t)nc;
}

void dsmc_counts(sf_ctx* ctx, int sid1, int sid2, double* count_sum, double* real_sum) {
  get_species(ctx, sid1);
  get_species(ctx, sid2);
  SfDsmcState* st = find_dsmc(ctx, sid1, sid2);
  SF_REQUIRE(st, SF_ERR_STATE, "no DSMC performed for this pair");
  SF_CUDA(cudaSetDevice(ctx->device));
  const int nc = ctx->ncells();
  std::vector<double2> h(nc);
  copy_wait(h.data(), st->counts, sizeof(double2) * nc, cudaMemcpyDeviceToHost, ctx->stream);
  for (int c = 0; c < nc; c++) {
    if (count_sum) count_sum[c] = h[c].x;
    if (real_sum) real_sum[c] = h[c].y;
  }
}

}  // namespace

extern "C" {

int sf_dsmc(sf_ctx* ctx, int32_t sid, const sf_sigma* sigma, double dt, double sig_cr_max0, int64_t* n_coll) {
  SF_API_BEGIN
  dsmc_run(ctx, sid, sid, sigma, nullptr, dt, sig_cr_max0, n_coll);
  SF_API_END(ctx)
}

int sf_dsmc_pair(sf_ctx* ctx, int32_t sid1, int32_t sid2, const sf_sigma* sigma1, const sf_sigma* sigma2, double dt,
                 double sig_cr_max0, int64_t* n_coll) {
  SF_API_BEGIN
  SF_REQUIRE(sid1 == sid2 || sigma2, SF_ERR_ARG, "a pair of two species needs the second material's sigma data");
  dsmc_run(ctx, sid1, sid2, sigma1, sigma2, dt, sig_cr_max0, n_coll);
  SF_API_END(ctx)
}

int sf_dsmc_get_counts(sf_ctx* ctx, int32_t sid, double* count_sum, double* real_sum) {
  SF_API_BEGIN
  dsmc_counts(ctx, sid, sid, count_sum, real_sum);
  SF_API_END(ctx)
}

int sf_dsmc_pair_get_counts(sf_ctx* ctx, int32_t sid1, int32_t sid2, double* count_sum, double* real_sum) {
  SF_API_BEGIN
  dsmc_counts(ctx, sid1, sid2, count_sum, real_sum);
  SF_API_END(ctx)
}

int sf_mcc_set_target(sf_ctx* ctx, double mass, const double* den, const double* u, const double* v, const double* w,
                      const double* temp) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && den && temp && mass > 0, SF_ERR_ARG, "target needs mass, density and temperature");
  SF_CUDA(cudaSetDevice(ctx->device));
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  if (!ctx->mcc_target) SF_CUDA(cudaMalloc(&ctx->mcc_target, sizeof(float) * 5 * nn));
  if (!ctx->mcc_sums) {
    SF_CUDA(cudaMalloc(&ctx->mcc_sums, sizeof(double) * 4 * nn));
    zero_wait(ctx->mcc_sums, sizeof(double) * 4 * nn, ctx->stream);
  }
  if (!ctx->mcc_cnt) SF_CUDA(cudaMalloc(&ctx->mcc_cnt, sizeof(unsigned long long) * 4));
  std::vector<float> h(5 * nn, 0.f);
  const double* src[5] = {den, u, v, w, temp};
  for (int k = 0; k < 5; k++)
    if (src[k])
      for (size_t q = 0; q < nn; q++) h[k * nn + q] = (float)src[k][q];
  copy_wait(ctx->mcc_target, h.data(), sizeof(float) * 5 * nn, cudaMemcpyHostToDevice, ctx->stream);
  ctx->mcc_mass = mass;
  SF_API_END(ctx)
}

namespace {

// One MCC.perform: the kernel over the source species, then the counts; the new
// electrons and ions (ionization) extend their species' slot ranges.
void mcc_run(sf_ctx* ctx, SfSpecies* sp, int model, const sf_sigma* sigma, double dt, SfSpecies* prod, double e_ion,
             unsigned long long out[3]) {
  SF_REQUIRE(ctx->mcc_target, SF_ERR_STATE, "no MCC target (sf_mcc_set_target)");
  SF_REQUIRE(dt > 0, SF_ERR_ARG, "dt must be positive");
  SF_CUDA(cudaSetDevice(ctx->device));
  const SigmaDev sg = make_sigma(sigma, nullptr, sp->mass, ctx->mcc_mass);
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  TargetView tg;
  tg.den = ctx->mcc_target;
  tg.u = ctx->mcc_target + nn;
  tg.v = ctx->mcc_target + 2 * nn;
  tg.w = ctx->mcc_target + 3 * nn;
  tg.T = ctx->mcc_target + 4 * nn;
  tg.mass = (float)ctx->mcc_mass;
  MccExtra ex{};
  ex.S = ctx->mcc_sums;
  ex.count_sum = ctx->mcc_sums + nn;
  ex.real_sum = ctx->mcc_sums + 2 * nn;
  ex.dn = ctx->mcc_sums + 3 * nn;
  ex.spwt = sp->spwt;
  ex.dt = dt;
  ex.Pe = sp->cur;
  ex.cap_e = sp->cap;
  if (prod) {
    ex.e_ion = e_ion;
    ex.prod_mass = prod->mass;
    ex.prod_spwt = prod->spwt;
    ex.spwt_ratio = sp->spwt / prod->spwt;
    ex.qm_halfdt_src = (float)(sp->charge / sp->mass * 0.5 * dt);
    ex.qm_halfdt_prod = (float)(prod->charge / prod->mass * 0.5 * dt);
    ex.Pi = prod->cur;
    ex.cap_i = prod->cap;
  }
  SF_CUDA(cudaMemsetAsync(ctx->mcc_cnt, 0, sizeof(unsigned long long) * 4, ctx->stream));
  if (sp->n > 0) {
    TimedScope ts(ctx, "mcc");
    k_mcc<<<grid_for(sp->n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
        ctx->mesh_view(), sp->cur, tg, sg, model, (float)sp->mass, (float)dt, ctx->seed ^ 0x3CC0ULL, ctx->rng_epoch++,
        ctx->mcc_cnt, ex);
    ctx->launches++;
  }
  SF_CUDA(cudaGetLastError());
  unsigned long long h[4] = {0, 0, 0, 0};
  SF_CUDA(cudaMemcpyAsync(h, ctx->mcc_cnt, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  timer_collect(ctx);
  if (prod) {
    const int64_t ne = std::min<int64_t>((int64_t)h[1], sp->cap - sp->n);
    const int64_t ni = std::min<int64_t>((int64_t)h[2], prod->cap - prod->n);
    sp->n += ne;
    sp->cur.n = sp->n;
    prod->n += ni;
    prod->cur.n = prod->n;
    if (ne > 0) sp->sorted = false;
    if (ni > 0) prod->sorted = false;
  }
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  SF_REQUIRE(h[3] == 0, SF_ERR_OOM, "MCC ionization products exceeded a species' capacity (the excess was dropped)");
}

}  // namespace

int sf_mcc(sf_ctx* ctx, int32_t sid, int32_t model, const sf_sigma* sigma, double dt, int64_t* n_coll) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(model == SF_MCC_MEX || model == SF_MCC_CEX, SF_ERR_ARG,
             "bad MCC model (ionization: sf_mcc_ionization)");
  unsigned long long h[3];
  mcc_run(ctx, sp, model, sigma, dt, nullptr, 0.0, h);
  if (n_coll) *n_coll = (int64_t)h[0];
  SF_API_END(ctx)
}

int sf_mcc_ionization(sf_ctx* ctx, int32_t sid, int32_t product_sid, const sf_sigma* sigma, double ionization_energy,
                      double dt, int64_t* n_coll, int64_t* n_electrons, int64_t* n_ions) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SfSpecies* prod = get_species(ctx, product_sid);
  SF_REQUIRE(product_sid != sid, SF_ERR_ARG, "the product (ion) species must differ from the source (electrons)");
  SF_REQUIRE(ionization_energy >= 0, SF_ERR_ARG, "ionization energy must be >= 0 eV");
  unsigned long long h[3];
  mcc_run(ctx, sp, SF_MCC_IONIZATION, sigma, dt, prod, ionization_energy, h);
  if (n_coll) *n_coll = (int64_t)h[0];
  if (n_electrons) *n_electrons = (int64_t)h[1];
  if (n_ions) *n_ions = (int64_t)h[2];
  SF_API_END(ctx)
}

int sf_mcc_get_sums(sf_ctx* ctx, double* S, double* count_sum, double* real_sum, double* delta_n, int32_t reset) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null context");
  SF_REQUIRE(ctx->mcc_sums, SF_ERR_STATE, "no MCC target (sf_mcc_set_target)");
  SF_CUDA(cudaSetDevice(ctx->device));
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  double* out[4] = {S, count_sum, real_sum, delta_n};
  for (int k = 0; k < 4; k++)
    if (out[k]) copy_wait(out[k], ctx->mcc_sums + k * nn, sizeof(double) * nn, cudaMemcpyDeviceToHost, ctx->stream);
  if (reset) zero_wait(ctx->mcc_sums, sizeof(double) * 4 * nn, ctx->stream);
  SF_API_END(ctx)
}

}  // extern "C"
