// sf_internal.h -- shared declarations of libstarfish_gpu.so (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/starfish_gpu.h"

namespace sf {

// ---------------------------------------------------------------------------------
// Errors: every ABI entry point catches sf::Error and turns it into a status code.
// ---------------------------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define SF_CUDA(x)                                                                    \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess)                                                            \
      throw ::sf::Error(e_ == cudaErrorMemoryAllocation ? SF_ERR_OOM : SF_ERR_CUDA,  \
                        std::string(#x) + ": " + cudaGetErrorString(e_));             \
  } while (0)

#define SF_REQUIRE(cond, code, msg)                          \
  do {                                                       \
    if (!(cond)) throw ::sf::Error((code), std::string(msg)); \
  } while (0)

constexpr uint32_t DEAD = 0xFFFFFFFFu;   // cell word of a removed particle
constexpr double QE = 1.60217646e-19;    // Constants.QE  (core/common/Constants.java:22)
constexpr double EPS0 = 8.85418782e-12;  // Constants.EPS0
constexpr double KB = 1.3806503e-23;     // Constants.K
constexpr double PI = 3.14159265358979323846;
constexpr double FLT_EPS_REF = 1e-7;     // Constants.FLT_EPS
// Deposit fixed point: one particle of weight spwt contributes S * 2^31 (S in [0,1]).
constexpr double DEP_SCALE = 2147483648.0;
// Moment fixed point: S * v * 2^16 per (m/s).
constexpr double MOM_SCALE = 65536.0;
// Second-moment fixed point (velocity sampling): S * v^2 * 2^4 per (m/s)^2.
constexpr double MOM2_SCALE = 16.0;

// Segment end points x1, y1, x2, y2 (16-byte aligned for vector loads).
struct alignas(16) Seg4 {
  double x, y, z, w;
};

// The same end points in cells from the mesh origin, split into an integer cell and an
// FP32 fraction: an end point relative to a cell is an exact integer difference plus one
// FP32 add (no FP64 work in the FP32 segment tests).
struct alignas(16) SegLC {
  int i1, j1, i2, j2;
  float f1, g1, f2, g2;
};

// Packed cell word: (j << 16) | i.  Meshes are limited to 65535 nodes per direction.
__host__ __device__ inline uint32_t pack_cell(int i, int j) { return ((uint32_t)j << 16) | (uint32_t)i; }
__host__ __device__ inline int cell_i(uint32_t c) { return (int)(c & 0xFFFFu); }
__host__ __device__ inline int cell_j(uint32_t c) { return (int)(c >> 16); }

// The FP32 electric field is stored per node u as (E[u], E[u+1]), so that the four corners
// of a cell are two 16-byte loads (u and u + ni) instead of four 8-byte ones.
// Bilinear gather at (i + fx, j + fy) (Field2D.gather, core/domain/Field2D.java:318-350).
__device__ __forceinline__ float2 gather_efield(const float4* __restrict__ E, int ni, int i, int j, float fx,
                                                float fy) {
  const int u = j * ni + i;
  const float4 lo = __ldg(E + u), hi = __ldg(E + u + ni);
  const float w00 = (1.f - fx) * (1.f - fy), w10 = fx * (1.f - fy), w11 = fx * fy, w01 = (1.f - fx) * fy;
  float2 e;
  e.x = w00 * lo.x + w10 * lo.z + w11 * hi.z + w01 * hi.x;
  e.y = w00 * lo.y + w10 * lo.w + w11 * hi.w + w01 * hi.y;
  return e;
}
// Asks L2 for `bytes` (a multiple of 16, from a 16-byte aligned address) with one bulk
// prefetch: a block issues it for its next chunk of particles while it works on the
// current one, so that the next chunk's loads find their lines in L2.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  if (bytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Writes node u's field into both of its places.
__device__ __forceinline__ void store_efield(float4* E, int u, float2 e) {
  reinterpret_cast<float2*>(E)[2 * (size_t)u] = e;
  if (u > 0) reinterpret_cast<float2*>(E)[2 * (size_t)u - 1] = e;
}
// Sort key of a cell: 16x16-cell tiles in row-major tile order, row-major inside a tile,
// so that a run of sorted particles is compact in both directions.
__host__ __device__ inline uint32_t cell_key(int i, int j, int ntx) {
  return ((uint32_t)((j >> 4) * ntx + (i >> 4)) << 8) | ((uint32_t)(j & 15) << 4) | (uint32_t)(i & 15);
}
__host__ __device__ inline void key_cell(uint32_t key, int ntx, int& i, int& j) {
  const int t = (int)(key >> 8);
  i = (t % ntx) * 16 + (int)(key & 15u);
  j = (t / ntx) * 16 + (int)((key >> 4) & 15u);
}

// ---------------------------------------------------------------------------------
// Device views (plain structs passed by value to kernels)
// ---------------------------------------------------------------------------------
struct MeshView {
  int ni, nj, nmax, domain;
  double x0[2], dh[2];
  double inv_dh[2];             // 1 / dh (the exact path multiplies: an FP64 division is ~10x dearer)
  float inv_dx, inv_dy;
  const float4* E;              // ni*nj: node u holds (efi, efj) of u and of u + 1, FP32
  const uint8_t* seg_dist;      // ni*nj Chebyshev distance to the nearest node listing a
                                // DIRICHLET/SINK segment (255 = none within 255)
  const uint8_t* seg_dist_tile; // per 16x16-node tile (row of (ni + 15) / 16): the least
                                // seg_dist of its nodes (a few KB, stays in L1)
  const int* node_seg_ptr;      // ni*nj+1
  const int* node_seg_idx;
  const Seg4* seg_xy;        // x1, y1, x2, y2
  const SegLC* seg_lc;       // the same end points in cells from the mesh origin
  const int* seg_btype;
  const int8_t* face_type;      // 4*nmax
  const double* node_vol;       // ni*nj
  int nseg;
  int all_delete;               // every domain face removes exiting particles
};

struct ProductView;

struct SurfaceView {
  const int* model;     // per segment SF_SURF_*
  const float4* param;  // vth, c_rest, c_accom, unused
  double* flux;         // 2 per segment
  double* deposit;      // 2 per segment
  const int2* product;  // per segment {product species or -1, vth of the product (float bits)}; null: none
  const ProductView* prod;  // by species index
};

struct ParticlesView {
  uint32_t* cell;
  float2* frac;
  float2* vxy;
  float* vz;
  int64_t n;  // slots in use
  float* w;   // per-slot weight as a fraction of the species weight (mpw / spwt, in (0, 1]);
              // null: every particle carries the species weight
};

// A species that surface impacts turn particles into (the ParticleListSource of the
// product material): its particles from slot P.n, counted in *added.
struct ProductView {
  ParticlesView P;
  int64_t cap;
  unsigned long long* added;
  double spwt;       // the product's (uniform) weight
  float qm_halfdt;   // (q/m) dt/2 of the addParticle rewind
  float vth;         // unused (the product's wall vth is per segment)
};

// Per-launch arguments of the push (sf_push.cu) and of its exact surface path.
struct PushArgs {
  float qm_dt;        // (q/m) dt
  float dt_dx, dt_dy; // dt/dx, dt/dy
  float dt;
  float dx, dy;
  float r0x, r0y;     // mesh origin (radius origin for RZ / ZR)
  double dt64;
  double qm;          // q/m
  double charge, spwt;
  uint64_t seed;
  uint32_t step;
};

struct SlowArgs {
  SurfaceView sv;
  unsigned long long* counters;
  double* stats_slow;   // 5 sums + boundary charge
  int stats;            // the totals (stats_slow) are wanted
};

// ---------------------------------------------------------------------------------
// Philox4x32-10 counter-based RNG (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11).  Streams are keyed by (seed, purpose) and
// counted by (particle or cell index, step, draw).
// ---------------------------------------------------------------------------------
struct Philox {
  uint4 ctr;
  uint2 key;
  uint4 buf;
  int left;
  __device__ Philox(uint64_t seed, uint32_t stream, uint64_t index, uint32_t step) {
    key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32) ^ (stream * 0x9E3779B9u));
    ctr = make_uint4((uint32_t)index, (uint32_t)(index >> 32), step, 0u);
    left = 0;
  }
  __device__ static inline void round1(uint4& c, const uint2 k) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  __device__ inline uint4 block() {
    uint4 c = ctr;
    uint2 k = key;
#pragma unroll
    for (int r = 0; r < 10; r++) {
      round1(c, k);
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
    ctr.w++;
    return c;
  }
  __device__ inline uint32_t next_u32() {
    if (left == 0) {
      buf = block();
      left = 4;
    }
    uint32_t v = (left == 4) ? buf.x : (left == 3) ? buf.y : (left == 2) ? buf.z : buf.w;
    left--;
    return v;
  }
  // uniform in [0,1) with 53 random bits (the 53-bit integer is formed in integer
  // arithmetic: one conversion on the FP64 pipe)
  __device__ inline uint64_t bits53() {
    const uint32_t a = next_u32() >> 5, b = next_u32() >> 6;
    return ((uint64_t)a << 26) | b;
  }
  __device__ inline double uniform() { return (double)bits53() * (1.0 / 9007199254740992.0); }
  // Utils.SampleMaxw1D(1) of the reference: sqrt(1/2) (sum of 12 uniforms - 6); the 12
  // 53-bit uniforms are summed exactly as integers and converted once
  __device__ inline double maxw1d_unit() {
    uint64_t s = 0;
    for (int k = 0; k < 12; k++) s += bits53();
    return 0.7071067811865476 * ((double)s * (1.0 / 9007199254740992.0) - 6.0);
  }
  // the same sampler from 24-bit uniforms in FP32 (for velocities stored as FP32 anyway):
  // the integer sum is exact and rounded once
  __device__ inline float maxw1d_unit_f() {
    uint32_t s = 0;
    for (int k = 0; k < 12; k++) s += next_u32() >> 8;
    return 0.70710678f * ((float)s * (1.0f / 16777216.0f) - 6.0f);
  }
  // uniform in [0,1) with 24 random bits
  __device__ inline float uniformf() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
};

__device__ inline void seg_intersect(const Seg4 s, const double p3[2], const double p4[2], double t[2]) {
  // LinearSegment.intersect + InfiniteLineIntersect (core/boundaries/LinearSegment.java:113-179)
  const double x1 = s.x, y1 = s.y, x2 = s.z, y2 = s.w;
  const double x3 = p3[0], y3 = p3[1], x4 = p4[0], y4 = p4[1];
  double den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
  if (den == 0) { t[0] = -1; t[1] = -1; return; }
  double xp0 = ((x1 * y2 - y1 * x2) * (x3 - x4) - (x1 - x2) * (x3 * y4 - y3 * x4)) / den;
  double xp1 = ((x1 * y2 - y1 * x2) * (y3 - y4) - (y1 - y2) * (x3 * y4 - y3 * x4)) / den;
  if (fabs(x2 - x1) > 1e-6) t[0] = (xp0 - x1) / (x2 - x1);
  else t[0] = (xp1 - y1) / (y2 - y1);
  if (t[0] < -FLT_EPS_REF || t[0] > (1 + FLT_EPS_REF)) { t[0] = -1; t[1] = -1; return; }
  if (fabs(x4 - x3) > 1e-6) t[1] = (xp0 - x3) / (x4 - x3);
  else t[1] = (xp1 - y3) / (y4 - y3);
  if (t[1] < -FLT_EPS_REF || t[1] > (1 + FLT_EPS_REF)) { t[0] = -1; t[1] = -1; return; }
  t[0] = fmin(fmax(t[0], 0.0), 1.0);
  t[1] = fmin(fmax(t[1], 0.0), 1.0);
}

// RNG stream identifiers
enum : uint32_t { RNG_SURFACE = 1, RNG_DSMC = 2, RNG_MCC = 3, RNG_INJECT = 4, RNG_DSMC_HEAVY = 5 };

}  // namespace sf

// ---------------------------------------------------------------------------------
// Host-side context
// ---------------------------------------------------------------------------------
// Per-step deposits of the velocity sampling (KineticMaterial.updateSamples): second
// moments and macroparticles per cell; null when the species is not sampled.
struct SampleView {
  unsigned long long* mom2;  // 3*ni*nj, S v^2 MOM2_SCALE
  unsigned* mpc;             // ni*nj, particles per cell at the cell's lower-left node
};

struct SfSpecies {
  double charge = 0, mass = 1, spwt = 1, nd_back = 0;
  int64_t cap = 0;
  int64_t n = 0;         // slots in use (alive + removed, until the next sort)
  int64_t n_dead = 0;    // removed slots among n
  // Device counters kept by the density epilogue of every push: [0] slots removed by
  // pushes whose counts the host has not read yet (folded into n_dead by settle_species),
  // [1] particle-steps pushed since the species was created.
  unsigned long long* acc = nullptr;
  bool acc_pending = false;  // a push that did not wait may have added to acc[0]
  bool sorted = false;   // slots are in cell order with no removed slots
  sf::ParticlesView cur{}, alt{};
  unsigned long long* count = nullptr;  // ni*nj fixed-point deposit
  long long* mom = nullptr;             // 3*ni*nj fixed-point moments
  double* nd = nullptr;                 // ni*nj number density
  double* nd_factor = nullptr;          // ni*nj spwt / 2^31 / V: count -> density
  double* uvw = nullptr;                // 3*ni*nj mean velocity
  bool moments_valid = false;
  int* seg_model = nullptr;
  float4* seg_param = nullptr;
  int2* seg_product = nullptr;  // per segment {product species or -1, product vth bits}; null until set
  bool has_products = false;
  double* flux = nullptr;     // 2*nseg
  double* deposit = nullptr;  // 2*nseg
  uint32_t step = 0;          // pushes done (RNG counter)
  int sort_interval = 16;     // automatic sort every N pushes (0 = never)
  int sort_qb = 3;            // automatic sort key: blocks of 2^sort_qb x 2^sort_qb cells
  bool weighted = false;      // per-particle weights held (cur.w / alt.w)
  int pushes_since_sort = 1 << 30;
  // velocity sampling (allocated by sf_samples_clear)
  SampleView smp{nullptr, nullptr};
  double* samp = nullptr;   // 8*ni*nj running sums: count, u, v, w, uu, vv, ww, mpc
  double* gas = nullptr;    // 10*ni*nj: nd-ave, u/v/w-ave, T, T1, T2, T3, p, mpc
  int64_t num_samples = 0;
};

// One instance of a batch (sf_batch.cu): everything the batched kernels need to push,
// inject and deposit for it without host values, so that a batch step is one CUDA graph.
// Particle counts live on the device (sf_batch's n_dev); P.n is not used.
struct BatchInst {
  sf::MeshView m;
  sf::ParticlesView P;
  sf::PushArgs a;                  // a.step is advanced on the device after every push
  sf::SlowArgs sa;                 // counters and slow-path sums of the instance's context
  unsigned long long* count;   // species deposit (fixed point)
  int* slow_idx;
  double* nd;
  const double* nd_factor;         // per node spwt / 2^31 / V (the species')
  double nd_back;
  // Maxwellian inlet (MaxwellianSource on one segment); src_on = 0: no source
  double sx1, sy1, sx2, sy2, snx, sny, v_th, v_drift, src_dt, mp_step;
  float qm_halfdt;
  int src_on;
  uint64_t src_seed;
  int64_t cap;
};

// Device state of a batch step shared by the batched kernels
struct BatchDev {
  BatchInst* insts;
  int n;
  int64_t* n_dev;      // slots in use per instance
  int64_t* dead_dev;   // removed slots among them (until the next sort)
  double* rem_dev;     // source remainders
  int64_t* num_dev;    // particles to inject this step
  int64_t* base_dev;   // first slot of this step's injection
  unsigned long long* added_dev;
  int64_t* tile_start; // n + 1: prefix of push tiles over the instances
  int64_t* chunk_start;  // n + 1: prefix of slow-queue chunks over the instances
  uint32_t* step_dev;  // batch step counter (RNG epoch of the sources)
  int* overflow;       // set when a source hit an instance's capacity
  int any_weighted;    // some instance's species carries per-particle weights
};
namespace sf {
// batched phases of one step, all on `stream` (sf_push.cu, sf_source.cu)
void batch_inject(const BatchDev& b, cudaStream_t stream, int num_sms);
void batch_push(const BatchDev& b, cudaStream_t stream, int num_sms, int blocks_per_sm, int slow_blocks_per_sm);
// batched field phase (sf_poisson.cu): rho, the nonlinear solve and E of every context on
// one stream, each stage one launch for all; results equal the contexts' own
// sf_update_rho + sf_poisson_nl + sf_efield bit for bit
struct BatchPoisson;
BatchPoisson* batch_poisson_create(sf_ctx* const* ctxs, int n, int num_sms, cudaStream_t stream);
void batch_poisson_destroy(BatchPoisson* bp);
// status[i]: 1 converged, 2 not converged, 3 diverged; returns the phase's time (ms)
float batch_poisson_step(BatchPoisson* bp, const sf_poisson_params& prm, const int* iters, sf_solve_stats* st,
                         int* status);
}  // namespace sf

struct SfPoisson;    // sf_poisson.cu
struct SfDsmcState;  // sf_collide.cu
struct SfUnet;       // sf_unet.cu

// CUDA-event timing of named kernels on the context stream
struct SfTimer {
  bool on = false;
  struct Rec {
    std::string name;
    double ms = 0;
    int64_t launches = 0;
  };
  std::vector<Rec> recs;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;  // rec index, events
  std::vector<cudaEvent_t> pool;
};

struct sf_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  std::string err;
  // mesh (host copies)
  int ni = 0, nj = 0, nmax = 0, domain = 0;
  double x0[2] = {0, 0}, dh[2] = {1, 1};
  std::vector<int8_t> node_type, face_type;
  std::vector<double> bc_value, node_vol;
  int nseg = 0;
  std::vector<double> seg_xy;
  std::vector<int> seg_btype;
  // device mesh
  float4* E = nullptr;  // see MeshView::E
  bool efield_set = false;
  bool all_delete = false;  // no SYMMETRY / PERIODIC face anywhere
  int ntx = 0, nty = 0;     // 16x16-cell tiles of the sort key
  int nkeys = 0;            // ntx*nty*256
  uint8_t* seg_dist = nullptr;
  uint8_t* seg_dist_tile = nullptr;
  int* node_seg_ptr = nullptr;
  int* node_seg_idx = nullptr;
  sf::Seg4* d_seg_xy = nullptr;
  sf::SegLC* d_seg_lc = nullptr;
  int* d_seg_btype = nullptr;
  int8_t* d_face_type = nullptr;
  double* d_node_vol = nullptr;
  // scratch
  int* slow_idx = nullptr;        // capacity = max species capacity
  int64_t slow_cap = 0;
  unsigned long long* counters = nullptr;  // [0] slow count, [1] removed, [2] bounce-limited
  double* stats_partial = nullptr;         // per-block partial sums
  int stats_blocks = 0;
  int* bins = nullptr;                     // (ncells+1) sort bins
  int* bins_tmp = nullptr;
  int* scan_blocks = nullptr;
  double* host_pinned = nullptr;           // small pinned staging area
  double* dscratch = nullptr;              // ni*nj FP64 scratch (field transfers)
  std::vector<SfSpecies*> species;
  // surface impacts that change species: the species views (refreshed per push) and
  // their append counters, allocated by the first sf_species_set_surface_product
  sf::ProductView* d_prod = nullptr;
  unsigned long long* d_prod_added = nullptr;
  SfPoisson* poisson = nullptr;
  SfUnet* unet = nullptr;          // learned warm start of the Poisson solve
  std::vector<SfDsmcState*> dsmc;  // per species DSMC cell state
  float* mcc_target = nullptr;     // MCC target density, u, v, w, T (5 * ni*nj)
  double mcc_mass = 0;
  double* mcc_sums = nullptr;      // MCC S, count sum, weight sum, delta-N (4 * ni*nj)
  unsigned long long* mcc_cnt = nullptr;  // collisions, new electrons, new ions (3)
  uint64_t seed = 0x5eed5eedULL;
  uint32_t rng_epoch = 0;  // advanced by every stochastic call (sources, DSMC, MCC)
  int64_t launches = 0;   // kernels launched
  SfTimer timer;

  sf::MeshView mesh_view() const;
  int ncells() const { return (ni - 1) * (nj - 1); }
};

// helpers shared between translation units
void sf_poisson_destroy_internal(sf_ctx* ctx);                       // sf_poisson.cu
void sf_collide_destroy_internal(sf_ctx* ctx);                       // sf_collide.cu
int sf_poisson_get_field_internal(sf_ctx* ctx, int field, double* out);  // sf_poisson.cu
void sf_unet_destroy_internal(sf_ctx* ctx);                          // sf_unet.cu
// Poisson hooks of the learned warm start (sf_unet.cu): phi <- phi_prev + prediction
// before a solve (false when the network cannot predict yet), and after a converged
// solve one training step on the new (d rho, d bc) -> d phi pair.
bool sf_unet_warm_start(sf_ctx* ctx, double* phi, const double* rho, const double* bc, const uint8_t* type);
void sf_unet_after_solve(sf_ctx* ctx, const double* phi, const double* rho, const double* bc,
                         const uint8_t* type, double eps);
// the prediction made the start worse: phi <- phi_prev (counted as rejected)
void sf_unet_reject(sf_ctx* ctx, double* phi);
// Coarse-correction mode of the network (sf_unet.cu): launches of the correction e of a
// linear residual r (returns the device buffer of e); the start of a solve (first
// residual, Newton diagonal, potential) kept for training; the training step after a
// converged solve; whether the network has been trained at all.
float* sf_unet_coarse_correction(sf_ctx* ctx, const float* r, const float* P, const uint8_t* type);
void sf_unet_coarse_start(sf_ctx* ctx, const float* r0, const float* P0, const double* phi0);
void sf_unet_coarse_train(sf_ctx* ctx, const double* phi_end, const uint8_t* type);
bool sf_unet_coarse_ready(const sf_ctx* ctx);
namespace sf {
// Counting sort of a species by cell key (sf_context.cu); with a look-ahead (cells per
// m/s in x and y) by the cell each particle reaches moving straight on, for locality only.
// Counting sort of a species' particles.  look_x/y: look-ahead in cells per (m/s) (0: the
// particles' current cells); qb: key blocks of 2^qb x 2^qb cells inside each 16x16-cell
// tile (0: exact cells, which binning by cell needs).  The automatic sort of the push passes
// the species' look-ahead and sort_qb.
void launch_sort(sf_ctx* ctx, SfSpecies* sp, float look_x = 0.f, float look_y = 0.f, int qb = 0);
void launch_finalize(sf_ctx* ctx, SfSpecies* sp, bool moments, const unsigned long long* counters);
// The species, with the removed-slot counts of pushes that did not wait folded into
// n_dead (waits for the context stream when there are any).
SfSpecies* get_species(sf_ctx* ctx, int sid);
// The species as it stands, without waiting (the push entry points).
SfSpecies* get_species_nowait(sf_ctx* ctx, int sid);
void settle_species(sf_ctx* ctx, SfSpecies* sp);
const void* mapped_host(const void* p);
void copy_to_host(sf_ctx* ctx, double* out, const double* src, size_t n);
void ensure_scratch(sf_ctx* ctx, int64_t particles);
// Timing scope: brackets the kernels launched inside with events when timing is on.
struct TimedScope {
  sf_ctx* ctx;
  int rec = -1;
  cudaEvent_t a = nullptr, b = nullptr;
  TimedScope(sf_ctx* c, const char* name);
  ~TimedScope();
};
void timer_collect(sf_ctx* ctx);  // after a stream sync: accumulate pending event pairs
inline int grid_for(int64_t n, int block, int max_blocks) {
  int64_t g = (n + block - 1) / block;
  if (g > max_blocks) g = max_blocks;
  if (g < 1) g = 1;
  return (int)g;
}
// Set-up copies and fills.  Every stream here is created with cudaStreamNonBlocking, and
// the plain cudaMemcpy / cudaMemset run on the legacy stream, which such streams do not
// wait for: a plain zero fill issued before an async copy could land after it.  These
// run on the owning stream and return once it is done, so host buffers may go at once.
inline void copy_wait(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  SF_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, s));
  SF_CUDA(cudaStreamSynchronize(s));
}
inline void zero_wait(void* p, size_t bytes, cudaStream_t s) {
  SF_CUDA(cudaMemsetAsync(p, 0, bytes, s));
  SF_CUDA(cudaStreamSynchronize(s));
}
}  // namespace sf

// Wraps an ABI body: converts exceptions into status codes and records the message.
#define SF_API_BEGIN try {
#define SF_API_END(ctx)                                      \
  }                                                          \
  catch (const sf::Error& e) {                               \
    if (ctx) (ctx)->err = e.what();                          \
    return e.code;                                           \
  }                                                          \
  catch (const std::exception& e) {                          \
    if (ctx) (ctx)->err = e.what();                          \
    return SF_ERR_ARG;                                       \
  }                                                          \
  return SF_OK;
