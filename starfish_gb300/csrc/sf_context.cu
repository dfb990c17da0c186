// sf_context.cu -- context, mesh set-up, species and particle storage, cell sort.
//
// Particle storage is structure-of-arrays and cell-sorted:
//   cell : uint32 packed (j << 16 | i) of the cell holding the particle, DEAD if removed
//   frac : float2 in-cell fractions (lc = i + fx, j + fy), the reference's Particle.lc
//   vxy  : float2 in-plane velocity, vz : float out-of-plane velocity
// i.e. 24 bytes per particle instead of the reference's ~150-200 byte Particle
// objects (core/materials/KineticMaterial.java:1207-1282).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "sf_internal.h"

using namespace sf;

static std::string g_create_error;

sf::MeshView sf_ctx::mesh_view() const {
  sf::MeshView m;
  m.ni = ni;
  m.nj = nj;
  m.nmax = nmax;
  m.domain = domain;
  m.x0[0] = x0[0];
  m.x0[1] = x0[1];
  m.dh[0] = dh[0];
  m.dh[1] = dh[1];
  m.inv_dh[0] = 1.0 / dh[0];
  m.inv_dh[1] = 1.0 / dh[1];
  m.inv_dx = (float)(1.0 / dh[0]);
  m.inv_dy = (float)(1.0 / dh[1]);
  m.E = E;
  m.seg_dist = seg_dist;
  m.seg_dist_tile = seg_dist_tile;
  m.node_seg_ptr = node_seg_ptr;
  m.node_seg_idx = node_seg_idx;
  m.seg_xy = d_seg_xy;
  m.seg_lc = d_seg_lc;
  m.seg_btype = d_seg_btype;
  m.face_type = d_face_type;
  m.node_vol = d_node_vol;
  m.nseg = nseg;
  m.all_delete = all_delete ? 1 : 0;
  return m;
}

namespace sf {

SfSpecies* get_species_nowait(sf_ctx* ctx, int sid) {
  SF_REQUIRE(ctx != nullptr, SF_ERR_ARG, "null context");
  SF_REQUIRE(sid >= 0 && sid < (int)ctx->species.size(), SF_ERR_ARG, "bad species id");
  return ctx->species[sid];
}

void settle_species(sf_ctx* ctx, SfSpecies* sp) {
  if (!sp->acc_pending) return;
  unsigned long long removed = 0;
  copy_wait(&removed, sp->acc, sizeof(removed), cudaMemcpyDeviceToHost, ctx->stream);
  SF_CUDA(cudaMemsetAsync(sp->acc, 0, sizeof(unsigned long long), ctx->stream));
  sp->n_dead += (int64_t)removed;
  if (removed > 0) sp->sorted = false;
  sp->acc_pending = false;
  timer_collect(ctx);
}

// The device address of a host buffer the GPU can read and write directly (pinned memory
// from cudaHostAlloc or cudaHostRegister), or null for any other pointer.
const void* mapped_host(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

__global__ void k_copy_f64(size_t n, const double* __restrict__ src, double* __restrict__ dst) {
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < n; u += (size_t)gridDim.x * blockDim.x)
    dst[u] = src[u];
}

// FP64 device array -> host (the caller waits for the stream): stored over the host link
// by a kernel when the host buffer is pinned, else a copy.
void copy_to_host(sf_ctx* ctx, double* out, const double* src, size_t n) {
  double* m = static_cast<double*>(const_cast<void*>(mapped_host(out)));
  if (m) {
    k_copy_f64<<<grid_for((int64_t)n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(n, src, m);
    ctx->launches++;
    SF_CUDA(cudaGetLastError());
  } else {
    SF_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  }
}

SfSpecies* get_species(sf_ctx* ctx, int sid) {
  SfSpecies* sp = get_species_nowait(ctx, sid);
  settle_species(ctx, sp);
  return sp;
}

// Node volumes of a uniform mesh with clipped control volumes (Mesh.nodeVol,
// core/domain/Mesh.java:998-1020 with controlVolumeLCs 656-744 and area 961-985).
static void compute_node_volumes(sf_ctx* c) {
  c->node_vol.assign((size_t)c->ni * c->nj, 0.0);
  for (int j = 0; j < c->nj; j++)
    for (int i = 0; i < c->ni; i++) {
      double il = std::max(i - 0.5, 0.0), ih = std::min(i + 0.5, (double)(c->ni - 1));
      double jl = std::max(j - 0.5, 0.0), jh = std::min(j + 0.5, (double)(c->nj - 1));
      double area = (ih - il) * c->dh[0] * (jh - jl) * c->dh[1];
      double v = area;
      if (c->domain == SF_DOMAIN_RZ) {
        double ir = (i == 0) ? 0.25 : (i == c->ni - 1) ? c->ni - 1.25 : (double)i;
        v = 2 * PI * area * (c->x0[0] + ir * c->dh[0]);
      } else if (c->domain == SF_DOMAIN_ZR) {
        double jr = (j == 0) ? 0.25 : (j == c->nj - 1) ? c->nj - 1.25 : (double)j;
        v = 2 * PI * area * (c->x0[1] + jr * c->dh[1]);
      }
      c->node_vol[(size_t)j * c->ni + i] = v;
    }
}

// Chebyshev distance of every node to the nearest node that lists a segment the push
// must test (DIRICHLET or SINK boundaries, KineticMaterial.java:508-515).  A particle
// whose move spans at most d cells from a node with distance > d + 1 cannot meet a
// candidate segment, which is the push's fast-path test.
static std::vector<uint8_t> segment_distance(const sf_ctx* c, const std::vector<int>& ptr,
                                             const std::vector<int>& idx) {
  const int ni = c->ni, nj = c->nj;
  const int INF = 255;
  std::vector<int> d((size_t)ni * nj, INF);
  for (int u = 0; u < ni * nj; u++)
    for (int k = ptr[u]; k < ptr[u + 1]; k++) {
      int bt = c->seg_btype[idx[k]];
      if (bt == SF_BT_DIRICHLET || bt == SF_BT_SINK) {
        d[u] = 0;
        break;
      }
    }
  // two-pass chamfer transform with unit weights on all 8 neighbours (exact Chebyshev)
  for (int j = 0; j < nj; j++)
    for (int i = 0; i < ni; i++) {
      int& v = d[(size_t)j * ni + i];
      for (int dj = -1; dj <= 0; dj++)
        for (int di = -1; di <= 1; di++) {
          if (dj == 0 && di >= 0) continue;
          int ii = i + di, jj = j + dj;
          if (ii < 0 || ii >= ni || jj < 0) continue;
          v = std::min(v, d[(size_t)jj * ni + ii] + 1);
        }
    }
  for (int j = nj - 1; j >= 0; j--)
    for (int i = ni - 1; i >= 0; i--) {
      int& v = d[(size_t)j * ni + i];
      for (int dj = 0; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++) {
          if (dj == 0 && di <= 0) continue;
          int ii = i + di, jj = j + dj;
          if (ii < 0 || ii >= ni || jj >= nj) continue;
          v = std::min(v, d[(size_t)jj * ni + ii] + 1);
        }
    }
  std::vector<uint8_t> out((size_t)ni * nj);
  for (size_t u = 0; u < out.size(); u++) out[u] = (uint8_t)std::min(d[u], INF);
  return out;
}

TimedScope::TimedScope(sf_ctx* c, const char* name) : ctx(c) {
  if (!ctx->timer.on) return;
  auto& recs = ctx->timer.recs;
  for (size_t k = 0; k < recs.size(); k++)
    if (recs[k].name == name) rec = (int)k;
  if (rec < 0) {
    recs.push_back({name, 0.0, 0});
    rec = (int)recs.size() - 1;
  }
  auto get = [&]() {
    cudaEvent_t e;
    if (!ctx->timer.pool.empty()) {
      e = ctx->timer.pool.back();
      ctx->timer.pool.pop_back();
    } else {
      SF_CUDA(cudaEventCreate(&e));
    }
    return e;
  };
  a = get();
  b = get();
  SF_CUDA(cudaEventRecord(a, ctx->stream));
}

TimedScope::~TimedScope() {
  if (rec < 0) return;
  cudaEventRecord(b, ctx->stream);
  ctx->timer.pending.push_back({rec, {a, b}});
}

void timer_collect(sf_ctx* ctx) {
  for (auto& p : ctx->timer.pending) {
    float ms = 0;
    if (cudaEventSynchronize(p.second.second) == cudaSuccess &&
        cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
      ctx->timer.recs[p.first].ms += ms;
      ctx->timer.recs[p.first].launches++;
    }
    ctx->timer.pool.push_back(p.second.first);
    ctx->timer.pool.push_back(p.second.second);
  }
  ctx->timer.pending.clear();
}

void ensure_scratch(sf_ctx* ctx, int64_t particles) {
  if (particles <= ctx->slow_cap) return;
  if (ctx->slow_idx) cudaFree(ctx->slow_idx);
  ctx->slow_idx = nullptr;
  SF_CUDA(cudaMalloc(&ctx->slow_idx, sizeof(int) * (size_t)std::max<int64_t>(particles, 1)));
  ctx->slow_cap = particles;
}

}  // namespace sf

// ---------------------------------------------------------------------------------
// kernels: particle upload / download / rewind / sort
// ---------------------------------------------------------------------------------
namespace {

// lc (FP64) -> packed cell + FP32 fractions.  lc is already clamped to [0, n-1].
__device__ __host__ inline void lc_to_cell(double lx, double ly, int ni, int nj, uint32_t& cell,
                                           float2& f) {
  int i = (int)lx, j = (int)ly;
  if (i > ni - 2) i = ni - 2;
  if (j > nj - 2) j = nj - 2;
  if (i < 0) i = 0;
  if (j < 0) j = 0;
  cell = pack_cell(i, j);
  f = make_float2((float)(lx - i), (float)(ly - j));
}

__global__ void k_upload(int n, const double* __restrict__ lc, const double* __restrict__ vel,
                         int ni, int nj, ParticlesView p, int64_t base) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t c;
  float2 f;
  lc_to_cell(lc[2 * k], lc[2 * k + 1], ni, nj, c, f);
  int64_t d = base + k;
  p.cell[d] = c;
  p.frac[d] = f;
  p.vxy[d] = make_float2((float)vel[3 * k], (float)vel[3 * k + 1]);
  p.vz[d] = (float)vel[3 * k + 2];
}

// Velocity rewind by -dt/2 (KineticMaterial.addParticle, KineticMaterial.java:776-796).
__global__ void k_rewind(MeshView m, ParticlesView p, int64_t base, int n, float qm_halfdt) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int64_t d = base + k;
  uint32_t c = p.cell[d];
  int i = cell_i(c), j = cell_j(c);
  float2 f = p.frac[d];
  const float2 e = gather_efield(m.E, m.ni, i, j, f.x, f.y);
  float2 v = p.vxy[d];
  v.x -= qm_halfdt * e.x;
  v.y -= qm_halfdt * e.y;
  p.vxy[d] = v;
}

// efi / efj may be the caller's pinned host buffers, read over the host link
__global__ void k_pack_efield(int nn, const double* __restrict__ efi, const double* __restrict__ efj,
                              float4* __restrict__ E) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nn; u += gridDim.x * blockDim.x)
    store_efield(E, u, make_float2((float)efi[u], (float)efj[u]));
}

// Counting sort by cell key.  Each block takes chunks of SORT_CHUNK particles and
// counts their keys in a shared-memory hash table (open addressing, linear probing;
// a chunk has at most SORT_CHUNK distinct keys and the table twice as many slots, so a
// probe always ends).  Global memory is then touched once per distinct key per chunk
// instead of once per particle.
constexpr int SORT_B = 256;
constexpr int SORT_IPT = 4;
constexpr int SORT_CHUNK = SORT_B * SORT_IPT;
constexpr int SORT_HBITS = 11;
constexpr int SORT_HSIZE = 1 << SORT_HBITS;  // 2048 >= 2 * SORT_CHUNK
constexpr unsigned EMPTY_KEY = 0xFFFFFFFFu;

__device__ inline unsigned hash_slot(unsigned key) { return (key * 2654435761u) >> (32 - SORT_HBITS); }

// returns the slot of key, inserting it if absent
__device__ inline unsigned hash_insert(unsigned* hkey, unsigned key) {
  unsigned s = hash_slot(key);
  for (int probe = 0; probe < SORT_HSIZE; probe++) {
    unsigned k = hkey[s];
    if (k == key) return s;
    if (k == EMPTY_KEY) {
      unsigned prev = atomicCAS(&hkey[s], EMPTY_KEY, key);
      if (prev == EMPTY_KEY || prev == key) return s;
    }
    s = (s + 1) & (SORT_HSIZE - 1);
  }
  return SORT_HSIZE;  // unreachable: the table has more slots than a chunk has keys
}

// Sort key of a particle: its cell's key, or with a look-ahead the key of the cell it will
// reach in tau steps moving straight on (ax = tau dt / dx cells per m/s), clamped to the
// mesh.  The look-ahead only orders particles for locality: a species sorted at the middle
// of the interval between two sorts stays twice as compact on average as one sorted by its
// current cells, since its particles spread from their predicted cell both before and
// after.  With qb > 0 the key is that of the 2^qb x 2^qb block of cells holding the cell
// (tile-major, then row-major blocks inside the 16x16 tile): a coarser key gives the
// scatter long runs per key (particles of one old block land in few new blocks) while a
// run of sorted particles stays as compact as with exact cells.  Binning that needs the
// exact cells (DSMC) sorts with qb = 0 and no look-ahead.
struct SortLook {
  float ax, ay;
  int imax, jmax;  // ni - 2, nj - 2
  int qb;          // log2 of the key block edge in cells (0..4)
};
__device__ __forceinline__ unsigned sort_key(uint32_t c, float2 f, float2 v, int ntx, const SortLook& L) {
  int i = cell_i(c), j = cell_j(c);
  if (L.ax != 0.f || L.ay != 0.f) {
    const float di = fminf(fmaxf(f.x + v.x * L.ax, -1e6f), 1e6f), dj = fminf(fmaxf(f.y + v.y * L.ay, -1e6f), 1e6f);
    i = min(max(i + (int)floorf(di), 0), L.imax);
    j = min(max(j + (int)floorf(dj), 0), L.jmax);
  }
  if (L.qb == 0) return cell_key(i, j, ntx);
  const int s = 4 - L.qb;
  const unsigned tile = (unsigned)((j >> 4) * ntx + (i >> 4));
  return (tile << (2 * s)) | ((unsigned)((j & 15) >> L.qb) << s) | (unsigned)((i & 15) >> L.qb);
}

// L2 prefetch of the chunk at `base` (whole 16-byte groups inside [0, p.n)) of the arrays
// a sort pass reads: the cells (what 0), also fraction and velocity (1), everything (2).
__device__ __forceinline__ void prefetch_chunk(const ParticlesView& p, int64_t base, int what) {
  if (threadIdx.x != 0 || base >= p.n) return;
  const uint32_t m = (uint32_t)min(p.n - base, (int64_t)SORT_CHUNK);
  prefetch_l2(p.cell + base, (m * 4u) & ~15u);
  if (what < 1) return;
  prefetch_l2(p.frac + base, (m * 8u) & ~15u);
  prefetch_l2(p.vxy + base, (m * 8u) & ~15u);
  if (what < 2) return;
  prefetch_l2(p.vz + base, (m * 4u) & ~15u);
  if (p.w) prefetch_l2(p.w + base, (m * 4u) & ~15u);
}

__global__ void __launch_bounds__(SORT_B) k_sort_hist(ParticlesView p, int ntx, int* bins, SortLook L) {
  __shared__ unsigned hkey[SORT_HSIZE];
  __shared__ unsigned hcnt[SORT_HSIZE];
  const bool look = L.ax != 0.f || L.ay != 0.f;
  const int64_t stride = (int64_t)gridDim.x * SORT_CHUNK;
  for (int64_t base = (int64_t)blockIdx.x * SORT_CHUNK; base < p.n; base += stride) {
    prefetch_chunk(p, base + stride, look ? 1 : 0);
    for (int q = threadIdx.x; q < SORT_HSIZE; q += SORT_B) {
      hkey[q] = EMPTY_KEY;
      hcnt[q] = 0u;
    }
    // all of a thread's loads are issued before the first is used (no load waits on the
    // cell word of another: removed slots read their fraction and velocity too)
    uint32_t c[SORT_IPT];
    float2 f[SORT_IPT], v[SORT_IPT];
#pragma unroll
    for (int k = 0; k < SORT_IPT; k++) {
      const int64_t q = base + k * SORT_B + threadIdx.x;
      c[k] = DEAD;
      f[k] = v[k] = make_float2(0.f, 0.f);
      if (q < p.n) {
        c[k] = __ldcs(&p.cell[q]);
        if (look) {
          f[k] = __ldcs(&p.frac[q]);
          v[k] = __ldcs(&p.vxy[q]);
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SORT_IPT; k++) {
      if (c[k] == DEAD) continue;
      const unsigned slot = hash_insert(hkey, sort_key(c[k], f[k], v[k], ntx, L));
      if (slot < SORT_HSIZE) atomicAdd(&hcnt[slot], 1u);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < SORT_HSIZE; q += SORT_B)
      if (hcnt[q]) atomicAdd(&bins[hkey[q]], (int)hcnt[q]);
    __syncthreads();
  }
}

// Scatter pass: the chunk is first regrouped in shared memory by key (chunk-local
// offsets from a scan of the per-key counts), then written out so that consecutive
// threads store consecutive slots of each key's run -- coalesced writes instead of one
// partial sector per particle.
constexpr size_t SORT_SCATTER_SMEM =
    (size_t)SORT_HSIZE * 3 * sizeof(unsigned) +
    (size_t)SORT_CHUNK * (sizeof(uint32_t) + sizeof(float2) + sizeof(float2) + sizeof(float) + sizeof(int));

// W: the species holds per-particle weights (staged and moved as well)
template <bool W>
__global__ void __launch_bounds__(SORT_B) k_sort_scatter(ParticlesView src, ParticlesView dst, int ntx, int* cursor,
                                                         SortLook L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* s_frac = reinterpret_cast<float2*>(smem_raw);
  float2* s_vxy = s_frac + SORT_CHUNK;
  unsigned* hkey = reinterpret_cast<unsigned*>(s_vxy + SORT_CHUNK);
  unsigned* hcnt = hkey + SORT_HSIZE;  // counts, then the key run's first output slot
  unsigned* hoff = hcnt + SORT_HSIZE;  // chunk-local offset of each key
  uint32_t* s_cell = hoff + SORT_HSIZE;
  float* s_vz = reinterpret_cast<float*>(s_cell + SORT_CHUNK);
  int* s_dst = reinterpret_cast<int*>(s_vz + SORT_CHUNK);
  float* s_w = reinterpret_cast<float*>(s_dst + SORT_CHUNK);  // weighted species only (larger launch)
  __shared__ int warp_tot[SORT_B / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int SPT = SORT_HSIZE / SORT_B;  // slots per thread in the scan
  const int64_t stride = (int64_t)gridDim.x * SORT_CHUNK;
  for (int64_t base = (int64_t)blockIdx.x * SORT_CHUNK; base < src.n; base += stride) {
    prefetch_chunk(src, base + stride, 2);
    for (int q = threadIdx.x; q < SORT_HSIZE; q += SORT_B) {
      hkey[q] = EMPTY_KEY;
      hcnt[q] = 0u;
    }
    __syncthreads();
    unsigned slot[SORT_IPT], rank[SORT_IPT];
    // the whole chunk is requested at once (the staging below then needs no second trip
    // to memory)
    uint32_t r_cell[SORT_IPT];
    float2 r_frac[SORT_IPT], r_vxy[SORT_IPT];
    float r_vz[SORT_IPT], r_w[SORT_IPT];
#pragma unroll
    for (int k = 0; k < SORT_IPT; k++) {
      const int64_t q = base + k * SORT_B + threadIdx.x;
      r_cell[k] = DEAD;
      r_w[k] = 1.f;
      if (q < src.n) {
        r_cell[k] = __ldcs(&src.cell[q]);
        r_frac[k] = __ldcs(&src.frac[q]);
        r_vxy[k] = __ldcs(&src.vxy[q]);
        r_vz[k] = __ldcs(&src.vz[q]);
        if (W) r_w[k] = __ldcs(&src.w[q]);
      }
    }
#pragma unroll
    for (int k = 0; k < SORT_IPT; k++) {
      const uint32_t c = r_cell[k];
      slot[k] = SORT_HSIZE;
      if (c == DEAD) continue;
      slot[k] = hash_insert(hkey, sort_key(c, r_frac[k], r_vxy[k], ntx, L));
      if (slot[k] < SORT_HSIZE) rank[k] = atomicAdd(&hcnt[slot[k]], 1u);
    }
    __syncthreads();
    // chunk-local offsets by an exclusive scan of the key counts, and each key's run in the
    // output reserved at the same time.  Thread t owns slots t, t + SORT_B, ...: consecutive
    // lanes touch consecutive slots (no bank conflicts).  The runs of different keys may sit
    // in any order in the staging buffer; only a key's particles have to be contiguous.
    unsigned cnt[SPT], run[SPT];
    unsigned tsum = 0;
#pragma unroll
    for (int q = 0; q < SPT; q++) {
      const int sidx = threadIdx.x + q * SORT_B;
      cnt[q] = hcnt[sidx];
      run[q] = 0u;
      if (cnt[q]) run[q] = (unsigned)atomicAdd(&cursor[hkey[sidx]], (int)cnt[q]);
      tsum += cnt[q];
    }
    unsigned x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = (int)x;
    __syncthreads();
    unsigned wpre = 0;
    for (int w = 0; w < wid; w++) wpre += (unsigned)warp_tot[w];
    unsigned off = wpre + x - tsum;
#pragma unroll
    for (int q = 0; q < SPT; q++) {
      const int sidx = threadIdx.x + q * SORT_B;
      hoff[sidx] = off;
      off += cnt[q];
      if (cnt[q]) hcnt[sidx] = run[q];  // hcnt becomes the run's first output slot
    }
    __syncthreads();
    // stage the chunk in key order
#pragma unroll
    for (int k = 0; k < SORT_IPT; k++) {
      if (slot[k] >= SORT_HSIZE) continue;
      const unsigned l = hoff[slot[k]] + rank[k];
      s_cell[l] = r_cell[k];
      s_frac[l] = r_frac[k];
      s_vxy[l] = r_vxy[k];
      s_vz[l] = r_vz[k];
      if (W) s_w[l] = r_w[k];
      s_dst[l] = (int)(hcnt[slot[k]] + rank[k]);
    }
    __syncthreads();
    // live particles in the chunk = sum of the warp totals of the scan
    unsigned nl = 0;
    for (int w = 0; w < SORT_B / 32; w++) nl += (unsigned)warp_tot[w];
    for (unsigned l = threadIdx.x; l < nl; l += SORT_B) {
      const int d = s_dst[l];
      dst.cell[d] = s_cell[l];
      dst.frac[d] = s_frac[l];
      dst.vxy[d] = s_vxy[l];
      dst.vz[d] = s_vz[l];
      if (W) dst.w[d] = s_w[l];
    }
    __syncthreads();
  }
}

// Exclusive scan of n ints in three passes (block scan, scan of block sums, add).
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

__device__ inline int block_exclusive_scan(int v, int* smem_warp, int& total) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = (lane < (int)(blockDim.x >> 5)) ? smem_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    smem_warp[lane] = w;
  }
  __syncthreads();
  int warp_prefix = (wid > 0) ? smem_warp[wid - 1] : 0;
  total = smem_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_tiles(const int* in, int* out, int n, int* block_sums) {
  __shared__ int sw[32];
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int pre = block_exclusive_scan(s, sw, total);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    if (base + k < n) out[base + k] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_single(int* data, int n) {
  // exclusive scan of a short array (n <= SCAN_TILE * 64) by one block, looping
  __shared__ int sw[32];
  int carry = 0;
  for (int64_t t0 = 0; t0 < n; t0 += SCAN_TILE) {
    int64_t base = t0 + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
      v[k] = (base + k < n) ? data[base + k] : 0;
      s += v[k];
    }
    int total;
    int pre = block_exclusive_scan(s, sw, total) + carry;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
      if (base + k < n) data[base + k] = pre;
      pre += v[k];
    }
    carry += total;
  }
}

__global__ void k_scan_add(int* out, int n, const int* block_sums) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int add = block_sums[blockIdx.x];
  for (int k = threadIdx.x; k < SCAN_TILE; k += blockDim.x)
    if (base + k < n) out[base + k] += add;
}

}  // namespace

namespace sf {

// bins[0..n) -> exclusive prefix sums in place (uses ctx->bins_tmp and scan_blocks)
static void exclusive_scan(sf_ctx* ctx, int* data, int n) {
  int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_tiles<<<tiles, SCAN_BLOCK, 0, ctx->stream>>>(data, ctx->bins_tmp, n, ctx->scan_blocks);
  k_scan_single<<<1, SCAN_BLOCK, 0, ctx->stream>>>(ctx->scan_blocks, tiles);
  k_scan_add<<<tiles, 256, 0, ctx->stream>>>(ctx->bins_tmp, n, ctx->scan_blocks);
  SF_CUDA(cudaMemcpyAsync(data, ctx->bins_tmp, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice,
                          ctx->stream));
}

void launch_sort(sf_ctx* ctx, SfSpecies* sp, float look_x, float look_y, int qb) {
  SF_REQUIRE(qb >= 0 && qb <= 4, SF_ERR_ARG, "sort key block out of range");
  const int nk = ctx->nkeys >> (2 * qb);  // keys of 2^qb x 2^qb-cell blocks
  const SortLook L{look_x, look_y, ctx->ni - 2, ctx->nj - 2, qb};
  TimedScope ts(ctx, "sort");
  SF_CUDA(cudaMemsetAsync(ctx->bins, 0, sizeof(int) * (size_t)(nk + 1), ctx->stream));
  if (sp->n > 0) {
    ctx->launches += 5;
    int g = grid_for((sp->n + SORT_CHUNK - 1) / SORT_CHUNK, 1, ctx->num_sms * 6);
    k_sort_hist<<<g, SORT_B, 0, ctx->stream>>>(sp->cur, ctx->ntx, ctx->bins, L);
    exclusive_scan(ctx, ctx->bins, nk + 1);  // bins[key] = first slot of the key, bins[nk] = total
    SF_CUDA(cudaMemcpyAsync(ctx->bins_tmp, ctx->bins, sizeof(int) * (size_t)(nk + 1),
                            cudaMemcpyDeviceToDevice, ctx->stream));
    ParticlesView dst = sp->alt;
    dst.n = sp->n;
    // per device and the same for every context (set-up threads may sort concurrently)
    SF_CUDA(cudaFuncSetAttribute(k_sort_scatter<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SORT_SCATTER_SMEM));
    SF_CUDA(cudaFuncSetAttribute(k_sort_scatter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(SORT_SCATTER_SMEM + sizeof(float) * SORT_CHUNK)));
    // 52 KB of shared memory and 64 registers per block: 4 blocks per SM
    const int gs = grid_for((sp->n + SORT_CHUNK - 1) / SORT_CHUNK, 1, ctx->num_sms * 4);
    if (sp->cur.w)
      k_sort_scatter<true><<<gs, SORT_B, SORT_SCATTER_SMEM + sizeof(float) * SORT_CHUNK, ctx->stream>>>(
          sp->cur, dst, ctx->ntx, ctx->bins_tmp, L);
    else
      k_sort_scatter<false><<<gs, SORT_B, SORT_SCATTER_SMEM, ctx->stream>>>(sp->cur, dst, ctx->ntx, ctx->bins_tmp, L);
    SF_CUDA(cudaGetLastError());
    int total = 0;
    SF_CUDA(cudaMemcpyAsync(&total, ctx->bins + nk, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    std::swap(sp->cur, sp->alt);
    sp->cur.n = total;
    sp->alt.n = 0;
    sp->n = total;
  }
  sp->n_dead = 0;
  // the compaction dropped every removed slot, including those of pushes not yet read
  SF_CUDA(cudaMemsetAsync(sp->acc, 0, sizeof(unsigned long long), ctx->stream));
  sp->acc_pending = false;
  sp->sorted = true;
  sp->pushes_since_sort = 0;
}

}  // namespace sf

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
extern "C" {

const char* sf_version(void) { return "starfish_gb300 0.1 (sm_103a)"; }

const char* sf_last_error(const sf_ctx* ctx) {
  if (!ctx) return g_create_error.c_str();
  return ctx->err.c_str();
}

int sf_ctx_create(const sf_mesh_desc* md, int device, sf_ctx** out) {
  sf_ctx* ctx = nullptr;
  try {
    SF_REQUIRE(md && out, SF_ERR_ARG, "null argument");
    SF_REQUIRE(md->ni >= 3 && md->nj >= 3 && md->ni <= 65535 && md->nj <= 65535, SF_ERR_ARG,
               "mesh must have 3..65535 nodes per direction");
    SF_REQUIRE(md->dh[0] > 0 && md->dh[1] > 0, SF_ERR_ARG, "mesh spacing must be positive");
    SF_REQUIRE(md->domain_type >= SF_DOMAIN_XY && md->domain_type <= SF_DOMAIN_ZR, SF_ERR_ARG,
               "bad domain type");
    SF_REQUIRE(md->node_type && md->face_type, SF_ERR_ARG, "node_type and face_type are required");
    SF_REQUIRE(md->n_segments >= 0, SF_ERR_ARG, "negative segment count");
    SF_REQUIRE(md->n_segments == 0 || (md->seg_xy && md->seg_btype), SF_ERR_ARG,
               "segments need seg_xy and seg_btype");
    SF_REQUIRE(md->n_segments == 0 || (md->node_seg_ptr && md->node_seg_idx), SF_ERR_ARG,
               "segments need the node_seg_ptr/node_seg_idx lists");
    int ndev = 0;
    SF_CUDA(cudaGetDeviceCount(&ndev));
    SF_REQUIRE(device >= 0 && device < ndev, SF_ERR_ARG, "bad CUDA device index");
    SF_CUDA(cudaSetDevice(device));
    ctx = new sf_ctx();
    ctx->device = device;
    SF_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
    SF_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->ni = md->ni;
    ctx->nj = md->nj;
    ctx->nmax = std::max(md->ni, md->nj);
    ctx->domain = md->domain_type;
    ctx->x0[0] = md->x0[0];
    ctx->x0[1] = md->x0[1];
    ctx->dh[0] = md->dh[0];
    ctx->dh[1] = md->dh[1];
    const size_t nn = (size_t)md->ni * md->nj;
    ctx->node_type.assign(md->node_type, md->node_type + nn);
    for (size_t u = 0; u < nn; u++) {
      int t = ctx->node_type[u];
      SF_REQUIRE(t == SF_NODE_OPEN || t == SF_NODE_DIRICHLET || t == SF_NODE_INTERNAL, SF_ERR_ARG,
                 "unsupported node type (INSULATOR nodes are not supported)");
    }
    ctx->face_type.assign(md->face_type, md->face_type + 4 * (size_t)ctx->nmax);
    ctx->all_delete = true;
    for (int f = 0; f < 4; f++) {
      const int len = (f == SF_FACE_LEFT || f == SF_FACE_RIGHT) ? md->nj : md->ni;
      for (int k = 0; k < len; k++) {
        const int t = ctx->face_type[(size_t)f * ctx->nmax + k];
        if (t == SF_DB_SYMMETRY || t == SF_DB_PERIODIC) ctx->all_delete = false;
      }
    }
    ctx->bc_value.assign(nn, 0.0);
    if (md->bc_value) std::copy(md->bc_value, md->bc_value + nn, ctx->bc_value.begin());
    if (md->node_vol) {
      ctx->node_vol.assign(md->node_vol, md->node_vol + nn);
    } else {
      compute_node_volumes(ctx);
    }
    ctx->nseg = md->n_segments;
    std::vector<int> ptr(nn + 1, 0), idx;
    if (ctx->nseg > 0) {
      ctx->seg_xy.assign(md->seg_xy, md->seg_xy + 4 * (size_t)ctx->nseg);
      ctx->seg_btype.assign(md->seg_btype, md->seg_btype + ctx->nseg);
      std::copy(md->node_seg_ptr, md->node_seg_ptr + nn + 1, ptr.begin());
      SF_REQUIRE(ptr[0] == 0, SF_ERR_ARG, "node_seg_ptr[0] must be 0");
      for (size_t u = 0; u < nn; u++) SF_REQUIRE(ptr[u + 1] >= ptr[u], SF_ERR_ARG, "node_seg_ptr not monotone");
      idx.assign(md->node_seg_idx, md->node_seg_idx + ptr[nn]);
      for (int s : idx) SF_REQUIRE(s >= 0 && s < ctx->nseg, SF_ERR_ARG, "node_seg_idx out of range");
    }
    std::vector<uint8_t> sd = segment_distance(ctx, ptr, idx);
    // device mesh
    SF_CUDA(cudaMalloc(&ctx->E, sizeof(float4) * nn));
    SF_CUDA(cudaMemsetAsync(ctx->E, 0, sizeof(float4) * nn, ctx->stream));
    SF_CUDA(cudaMalloc(&ctx->seg_dist, nn));
    copy_wait(ctx->seg_dist, sd.data(), nn, cudaMemcpyHostToDevice, ctx->stream);
    {
      const int tx = (ctx->ni + 15) / 16, ty = (ctx->nj + 15) / 16;
      std::vector<uint8_t> st((size_t)tx * ty, 255);
      for (int j = 0; j < ctx->nj; j++)
        for (int i = 0; i < ctx->ni; i++) {
          uint8_t& t = st[(size_t)(j >> 4) * tx + (i >> 4)];
          t = std::min(t, sd[(size_t)j * ctx->ni + i]);
        }
      SF_CUDA(cudaMalloc(&ctx->seg_dist_tile, st.size()));
      copy_wait(ctx->seg_dist_tile, st.data(), st.size(), cudaMemcpyHostToDevice, ctx->stream);
    }
    SF_CUDA(cudaMalloc(&ctx->node_seg_ptr, sizeof(int) * (nn + 1)));
    copy_wait(ctx->node_seg_ptr, ptr.data(), sizeof(int) * (nn + 1), cudaMemcpyHostToDevice, ctx->stream);
    SF_CUDA(cudaMalloc(&ctx->node_seg_idx, sizeof(int) * std::max<size_t>(idx.size(), 1)));
    if (!idx.empty())
      copy_wait(ctx->node_seg_idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, ctx->stream);
    SF_CUDA(cudaMalloc(&ctx->d_seg_xy, sizeof(Seg4) * std::max(ctx->nseg, 1)));
    SF_CUDA(cudaMalloc(&ctx->d_seg_lc, sizeof(SegLC) * std::max(ctx->nseg, 1)));
    SF_CUDA(cudaMalloc(&ctx->d_seg_btype, sizeof(int) * std::max(ctx->nseg, 1)));
    if (ctx->nseg > 0) {
      copy_wait(ctx->d_seg_xy, ctx->seg_xy.data(), sizeof(Seg4) * ctx->nseg, cudaMemcpyHostToDevice, ctx->stream);
      std::vector<SegLC> lcs(ctx->nseg);
      for (int s = 0; s < ctx->nseg; s++) {
        int ib[4];
        float fr[4];
        for (int q = 0; q < 4; q++) {
          const double l = (ctx->seg_xy[4 * (size_t)s + q] - ctx->x0[q & 1]) / ctx->dh[q & 1];
          const double b = std::floor(l);
          ib[q] = (int)b;
          fr[q] = (float)(l - b);
        }
        lcs[s] = SegLC{ib[0], ib[1], ib[2], ib[3], fr[0], fr[1], fr[2], fr[3]};
      }
      copy_wait(ctx->d_seg_lc, lcs.data(), sizeof(SegLC) * ctx->nseg, cudaMemcpyHostToDevice, ctx->stream);
      copy_wait(ctx->d_seg_btype, ctx->seg_btype.data(), sizeof(int) * ctx->nseg, cudaMemcpyHostToDevice, ctx->stream);
    }
    SF_CUDA(cudaMalloc(&ctx->d_face_type, 4 * (size_t)ctx->nmax));
    copy_wait(ctx->d_face_type, ctx->face_type.data(), 4 * (size_t)ctx->nmax, cudaMemcpyHostToDevice, ctx->stream);
    SF_CUDA(cudaMalloc(&ctx->d_node_vol, sizeof(double) * nn));
    copy_wait(ctx->d_node_vol, ctx->node_vol.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, ctx->stream);
    SF_CUDA(cudaMalloc(&ctx->counters, sizeof(unsigned long long) * 8));
    ctx->stats_blocks = ctx->num_sms * 8;
    SF_CUDA(cudaMalloc(&ctx->stats_partial, sizeof(double) * 8 * (size_t)ctx->stats_blocks));
    ctx->ntx = (ctx->ni - 1 + 15) / 16;
    ctx->nty = (ctx->nj - 1 + 15) / 16;
    ctx->nkeys = ctx->ntx * ctx->nty * 256;
    int nk = ctx->nkeys;
    SF_CUDA(cudaMalloc(&ctx->bins, sizeof(int) * (size_t)(nk + 1)));
    SF_CUDA(cudaMalloc(&ctx->bins_tmp, sizeof(int) * (size_t)(nk + 1)));
    SF_CUDA(cudaMalloc(&ctx->scan_blocks, sizeof(int) * (size_t)((nk + 1) / SCAN_TILE + 2)));
    SF_CUDA(cudaMallocHost(&ctx->host_pinned, sizeof(double) * 64));
    SF_CUDA(cudaMalloc(&ctx->dscratch, sizeof(double) * nn * 2));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = ctx;
    return SF_OK;
  } catch (const sf::Error& e) {
    g_create_error = e.what();
    if (ctx) sf_ctx_destroy(ctx);
    return e.code;
  } catch (const std::exception& e) {
    g_create_error = e.what();
    if (ctx) sf_ctx_destroy(ctx);
    return SF_ERR_ARG;
  }
}

// Starfish.random (core/common/Starfish.java:238, reseeded by <starfish randomize> at
// :647): the seed of every random stream of the context (sources, surfaces, DSMC, MCC).
int sf_ctx_set_seed(sf_ctx* ctx, uint64_t seed) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null context");
  ctx->seed = seed;
  ctx->rng_epoch = 0;
  for (SfSpecies* sp : ctx->species) sp->step = 0;
  SF_API_END(ctx)
}

int sf_ctx_destroy(sf_ctx* ctx) {
  if (!ctx) return SF_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  sf_unet_destroy_internal(ctx);
  sf_poisson_destroy_internal(ctx);
  sf_collide_destroy_internal(ctx);
  for (SfSpecies* sp : ctx->species) {
    void* ptrs[] = {sp->cur.cell, sp->cur.frac, sp->cur.vxy,  sp->cur.vz,     sp->alt.cell,  sp->alt.frac,
                    sp->alt.vxy,  sp->alt.vz,   sp->count,    sp->mom,        sp->nd,        sp->uvw,
                    sp->seg_model, sp->seg_param, sp->flux,   sp->deposit,    sp->smp.mom2,  sp->smp.mpc,
                    sp->samp,     sp->gas,      sp->seg_product, sp->cur.w,   sp->alt.w,
                    sp->acc,      sp->nd_factor};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    delete sp;
  }
  void* ptrs[] = {ctx->E, ctx->seg_dist, ctx->seg_dist_tile, ctx->node_seg_ptr, ctx->node_seg_idx, ctx->d_seg_xy, ctx->d_seg_lc,
                  ctx->d_seg_btype, ctx->d_face_type, ctx->d_node_vol, ctx->slow_idx, ctx->counters,
                  ctx->stats_partial, ctx->bins, ctx->bins_tmp, ctx->scan_blocks, ctx->dscratch};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (ctx->d_prod) cudaFree(ctx->d_prod);
  if (ctx->d_prod_added) cudaFree(ctx->d_prod_added);
  if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
  for (auto& p : ctx->timer.pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  for (cudaEvent_t e : ctx->timer.pool) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SF_OK;
}

int sf_species_add(sf_ctx* ctx, double charge, double mass, double spwt, int64_t capacity,
                   double nd_back, int32_t* sid) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && sid, SF_ERR_ARG, "null argument");
  SF_REQUIRE(mass > 0 && spwt > 0, SF_ERR_ARG, "mass and spwt must be positive");
  SF_REQUIRE(capacity > 0 && capacity < (int64_t)1 << 31, SF_ERR_ARG, "capacity must be in (0, 2^31)");
  SF_CUDA(cudaSetDevice(ctx->device));
  SfSpecies* sp = new SfSpecies();
  ctx->species.push_back(sp);  // owned by the context from here on (freed on destroy)
  sp->charge = charge;
  sp->mass = mass;
  sp->spwt = spwt;
  sp->nd_back = nd_back;
  sp->cap = capacity;
  const size_t nn = (size_t)ctx->ni * ctx->nj;
  for (ParticlesView* pv : {&sp->cur, &sp->alt}) {
    SF_CUDA(cudaMalloc(&pv->cell, sizeof(uint32_t) * (size_t)capacity));
    SF_CUDA(cudaMalloc(&pv->frac, sizeof(float2) * (size_t)capacity));
    SF_CUDA(cudaMalloc(&pv->vxy, sizeof(float2) * (size_t)capacity));
    SF_CUDA(cudaMalloc(&pv->vz, sizeof(float) * (size_t)capacity));
    pv->n = 0;
  }
  SF_CUDA(cudaMalloc(&sp->count, sizeof(unsigned long long) * nn));
  SF_CUDA(cudaMemsetAsync(sp->count, 0, sizeof(unsigned long long) * nn, ctx->stream));
  SF_CUDA(cudaMalloc(&sp->acc, sizeof(unsigned long long) * 2));
  SF_CUDA(cudaMemsetAsync(sp->acc, 0, sizeof(unsigned long long) * 2, ctx->stream));
  SF_CUDA(cudaMalloc(&sp->mom, sizeof(long long) * 3 * nn));
  SF_CUDA(cudaMalloc(&sp->nd, sizeof(double) * nn));
  SF_CUDA(cudaMemsetAsync(sp->nd, 0, sizeof(double) * nn, ctx->stream));
  {
    // the density epilogue's factor per node: one FP64 multiply-add per node instead of a
    // divide (an FP64 divide is a dozen FP64-pipe instructions)
    std::vector<double> f(nn);
    const double w_scale = spwt / DEP_SCALE;
    for (size_t u = 0; u < nn; u++) f[u] = w_scale * (1.0 / ctx->node_vol[u]);
    SF_CUDA(cudaMalloc(&sp->nd_factor, sizeof(double) * nn));
    copy_wait(sp->nd_factor, f.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, ctx->stream);
  }
  SF_CUDA(cudaMalloc(&sp->uvw, sizeof(double) * 3 * nn));
  SF_CUDA(cudaMemsetAsync(sp->uvw, 0, sizeof(double) * 3 * nn, ctx->stream));
  int ns = std::max(ctx->nseg, 1);
  std::vector<int> model(ns, SF_SURF_ABSORB);
  std::vector<float4> param(ns, make_float4(0, 1, 1, 0));
  SF_CUDA(cudaMalloc(&sp->seg_model, sizeof(int) * ns));
  copy_wait(sp->seg_model, model.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, ctx->stream);
  SF_CUDA(cudaMalloc(&sp->seg_param, sizeof(float4) * ns));
  copy_wait(sp->seg_param, param.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, ctx->stream);
  SF_CUDA(cudaMalloc(&sp->flux, sizeof(double) * 2 * ns));
  SF_CUDA(cudaMalloc(&sp->deposit, sizeof(double) * 2 * ns));
  SF_CUDA(cudaMemsetAsync(sp->flux, 0, sizeof(double) * 2 * ns, ctx->stream));
  SF_CUDA(cudaMemsetAsync(sp->deposit, 0, sizeof(double) * 2 * ns, ctx->stream));
  ensure_scratch(ctx, capacity);
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  *sid = (int32_t)ctx->species.size() - 1;
  SF_API_END(ctx)
}

int sf_species_set_surface(sf_ctx* ctx, int32_t sid, int32_t seg, int32_t model, double vth,
                           double c_rest, double c_accom) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(seg >= 0 && seg < ctx->nseg, SF_ERR_ARG, "bad segment index");
  SF_REQUIRE(model >= SF_SURF_PASS && model <= SF_SURF_DIFFUSE, SF_ERR_ARG, "bad surface model");
  SF_REQUIRE(model != SF_SURF_DIFFUSE || vth > 0, SF_ERR_ARG, "DIFFUSE needs vth > 0");
  float4 p = make_float4((float)vth, (float)c_rest, (float)c_accom, 0.f);
  copy_wait(sp->seg_model + seg, &model, sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
  copy_wait(sp->seg_param + seg, &p, sizeof(float4), cudaMemcpyHostToDevice, ctx->stream);
  SF_API_END(ctx)
}

int sf_species_set_surface_product(sf_ctx* ctx, int32_t sid, int32_t seg, int32_t product_sid, double vth_product) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(seg >= 0 && seg < ctx->nseg, SF_ERR_ARG, "bad segment index");
  SF_REQUIRE(product_sid == -1 || (product_sid >= 0 && product_sid < (int)ctx->species.size()), SF_ERR_ARG,
             "bad product species");
  SF_REQUIRE(product_sid != sid, SF_ERR_ARG, "the product must differ from the impacting species");
  SF_REQUIRE(product_sid < 0 || vth_product >= 0, SF_ERR_ARG, "vth_product must be >= 0");
  SF_REQUIRE(ctx->species.size() <= 64, SF_ERR_ARG, "at most 64 species with surface products");
  SF_CUDA(cudaSetDevice(ctx->device));
  const int ns = std::max(ctx->nseg, 1);
  if (!sp->seg_product) {
    SF_CUDA(cudaMalloc(&sp->seg_product, sizeof(int2) * ns));
    std::vector<int2> none(ns, make_int2(-1, 0));
    copy_wait(sp->seg_product, none.data(), sizeof(int2) * ns, cudaMemcpyHostToDevice, ctx->stream);
  }
  if (!ctx->d_prod) {
    SF_CUDA(cudaMalloc(&ctx->d_prod, sizeof(ProductView) * 64));
    SF_CUDA(cudaMalloc(&ctx->d_prod_added, sizeof(unsigned long long) * 64));
  }
  const float v = (float)vth_product;
  int vb;
  std::memcpy(&vb, &v, sizeof(vb));
  const int2 e = make_int2(product_sid, vb);
  copy_wait(sp->seg_product + seg, &e, sizeof(int2), cudaMemcpyHostToDevice, ctx->stream);
  if (product_sid >= 0) sp->has_products = true;
  SF_API_END(ctx)
}

// Shared body of the two append entry points: lc (n*2) and vel (n*3) on the host.
// mpw: per-particle weights (weighted species), or null for the species weight
static void append_lc_impl(sf_ctx* ctx, SfSpecies* sp, int64_t n, const double* lc, const double* vel,
                           bool rewind, double dt, const double* mpw = nullptr) {
  SF_REQUIRE(sp->n + n <= sp->cap, SF_ERR_OOM, "species capacity exceeded");
  if (sp->weighted) {
    // relative weights mpw / spwt in (0, 1]: the species weight bounds its particles'
    std::vector<float> w((size_t)n, 1.f);
    for (int64_t k = 0; mpw && k < n; k++) {
      const double r = mpw[k] / sp->spwt;
      SF_REQUIRE(r > 0.0 && r <= 1.0, SF_ERR_ARG, "particle weights must lie in (0, spwt]");
      w[(size_t)k] = (float)r;
    }
    copy_wait(sp->cur.w + sp->n, w.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
  }
  const int64_t CH = 1 << 22;
  double *dlc = nullptr, *dvel = nullptr;
  SF_CUDA(cudaMalloc(&dlc, sizeof(double) * 2 * (size_t)std::min(n, CH)));
  SF_CUDA(cudaMalloc(&dvel, sizeof(double) * 3 * (size_t)std::min(n, CH)));
  try {
    for (int64_t off = 0; off < n; off += CH) {
      int m = (int)std::min(CH, n - off);
      SF_CUDA(cudaMemcpyAsync(dlc, lc + 2 * off, sizeof(double) * 2 * m, cudaMemcpyHostToDevice, ctx->stream));
      SF_CUDA(cudaMemcpyAsync(dvel, vel + 3 * off, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, ctx->stream));
      k_upload<<<(m + 255) / 256, 256, 0, ctx->stream>>>(m, dlc, dvel, ctx->ni, ctx->nj, sp->cur, sp->n + off);
      ctx->launches++;
      if (rewind) {
        float qmh = (float)(sp->charge / sp->mass * 0.5 * dt);
        k_rewind<<<(m + 255) / 256, 256, 0, ctx->stream>>>(ctx->mesh_view(), sp->cur, sp->n + off, m, qmh);
        ctx->launches++;
      }
      SF_CUDA(cudaGetLastError());
    }
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    cudaFree(dlc);
    cudaFree(dvel);
    throw;
  }
  cudaFree(dlc);
  cudaFree(dvel);
  sp->n += n;
  sp->cur.n = sp->n;
  sp->sorted = false;
}

int sf_particles_append(sf_ctx* ctx, int32_t sid, int64_t n, const double* pos, const double* vel,
                        const double* mpw, int32_t rewind, double dt) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(n >= 0 && (n == 0 || (pos && vel)), SF_ERR_ARG, "null particle arrays");
  SF_REQUIRE(!rewind || ctx->efield_set, SF_ERR_STATE, "rewind needs the electric field");
  if (mpw && !sp->weighted)
    for (int64_t k = 0; k < n; k++)
      SF_REQUIRE(mpw[k] == sp->spwt, SF_ERR_ARG,
                 "per-particle weights that differ from the species spwt need sf_species_set_weighted");
  SF_CUDA(cudaSetDevice(ctx->device));
  // XtoL (UniformMesh.java:154-161) and the edge clamp of addParticle (KineticMaterial.java:764-772);
  // positions outside the mesh are rejected like Starfish.domain_module.getMesh(pos) == null.
  std::vector<double> lc(2 * (size_t)n);
  std::vector<double> v(3 * (size_t)n);
  std::vector<double> wk(mpw ? (size_t)n : 0);
  int64_t kept = 0;
  for (int64_t k = 0; k < n; k++) {
    double lx = (pos[3 * k] - ctx->x0[0]) / ctx->dh[0];
    double ly = (pos[3 * k + 1] - ctx->x0[1]) / ctx->dh[1];
    if (!(lx >= 0 && ly >= 0 && lx <= ctx->ni - 1 && ly <= ctx->nj - 1)) continue;
    lc[2 * kept] = lx;
    lc[2 * kept + 1] = ly;
    v[3 * kept] = vel[3 * k];
    v[3 * kept + 1] = vel[3 * k + 1];
    v[3 * kept + 2] = vel[3 * k + 2];
    if (mpw) wk[(size_t)kept] = mpw[k];
    kept++;
  }
  if (kept > 0) append_lc_impl(ctx, sp, kept, lc.data(), v.data(), rewind != 0, dt, mpw ? wk.data() : nullptr);
  SF_API_END(ctx)
}

int sf_particles_append_lc(sf_ctx* ctx, int32_t sid, int64_t n, const double* lc, const double* vel) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(n >= 0 && (n == 0 || (lc && vel)), SF_ERR_ARG, "null particle arrays");
  for (int64_t k = 0; k < n; k++)
    SF_REQUIRE(lc[2 * k] >= 0 && lc[2 * k + 1] >= 0 && lc[2 * k] <= ctx->ni - 1 && lc[2 * k + 1] <= ctx->nj - 1,
               SF_ERR_ARG, "logical coordinate outside the mesh");
  SF_CUDA(cudaSetDevice(ctx->device));
  if (n > 0) append_lc_impl(ctx, sp, n, lc, vel, false, 0.0);
  SF_API_END(ctx)
}

int sf_particles_append_lc_w(sf_ctx* ctx, int32_t sid, int64_t n, const double* lc, const double* vel,
                             const double* mpw) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(n >= 0 && (n == 0 || (lc && vel && mpw)), SF_ERR_ARG, "null particle arrays");
  SF_REQUIRE(sp->weighted, SF_ERR_STATE, "the species holds no per-particle weights (sf_species_set_weighted)");
  for (int64_t k = 0; k < n; k++)
    SF_REQUIRE(lc[2 * k] >= 0 && lc[2 * k + 1] >= 0 && lc[2 * k] <= ctx->ni - 1 && lc[2 * k + 1] <= ctx->nj - 1,
               SF_ERR_ARG, "logical coordinate outside the mesh");
  SF_CUDA(cudaSetDevice(ctx->device));
  if (n > 0) append_lc_impl(ctx, sp, n, lc, vel, false, 0.0, mpw);
  SF_API_END(ctx)
}

int sf_species_set_weighted(sf_ctx* ctx, int32_t sid, int32_t on) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(sp->n == 0, SF_ERR_STATE, "per-particle weights are switched before the first particle");
  SF_CUDA(cudaSetDevice(ctx->device));
  if (on && !sp->weighted) {
    SF_CUDA(cudaMalloc(&sp->cur.w, sizeof(float) * (size_t)std::max<int64_t>(sp->cap, 1)));
    SF_CUDA(cudaMalloc(&sp->alt.w, sizeof(float) * (size_t)std::max<int64_t>(sp->cap, 1)));
  } else if (!on && sp->weighted) {
    SF_CUDA(cudaFree(sp->cur.w));
    SF_CUDA(cudaFree(sp->alt.w));
    sp->cur.w = sp->alt.w = nullptr;
  }
  sp->weighted = on != 0;
  SF_API_END(ctx)
}

int sf_particles_download_weights(sf_ctx* ctx, int32_t sid, int64_t cap, double* mpw, int64_t* n_out) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(n_out, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaSetDevice(ctx->device));
  size_t n = (size_t)sp->n;
  std::vector<uint32_t> cell(n);
  std::vector<float> w(n, 1.f);
  if (n) {
    SF_CUDA(cudaMemcpyAsync(cell.data(), sp->cur.cell, 4 * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (sp->weighted) SF_CUDA(cudaMemcpyAsync(w.data(), sp->cur.w, 4 * n, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  int64_t k2 = 0;
  for (size_t k = 0; k < n; k++) {
    if (cell[k] == DEAD) continue;
    if (mpw && k2 < cap) mpw[k2] = (double)w[k] * sp->spwt;
    k2++;
  }
  *n_out = std::min(k2, cap);
  SF_REQUIRE(k2 <= cap, SF_ERR_ARG, "host arrays too small for the particle count");
  SF_API_END(ctx)
}

int sf_particles_count(sf_ctx* ctx, int32_t sid, int64_t* np) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(np, SF_ERR_ARG, "null argument");
  *np = sp->n - sp->n_dead;
  SF_API_END(ctx)
}

int sf_particles_download(sf_ctx* ctx, int32_t sid, int64_t cap, double* lc, double* vel, int64_t* n_out) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(n_out, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaSetDevice(ctx->device));
  size_t n = (size_t)sp->n;
  std::vector<uint32_t> cell(n);
  std::vector<float2> frac(n), vxy(n);
  std::vector<float> vz(n);
  if (n) {
    SF_CUDA(cudaMemcpyAsync(cell.data(), sp->cur.cell, 4 * n, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaMemcpyAsync(frac.data(), sp->cur.frac, 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaMemcpyAsync(vxy.data(), sp->cur.vxy, 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaMemcpyAsync(vz.data(), sp->cur.vz, 4 * n, cudaMemcpyDeviceToHost, ctx->stream));
    SF_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  int64_t w = 0;
  for (size_t k = 0; k < n; k++) {
    if (cell[k] == DEAD) continue;
    if (w < cap) {
      if (lc) {
        lc[2 * w] = cell_i(cell[k]) + (double)frac[k].x;
        lc[2 * w + 1] = cell_j(cell[k]) + (double)frac[k].y;
      }
      if (vel) {
        vel[3 * w] = vxy[k].x;
        vel[3 * w + 1] = vxy[k].y;
        vel[3 * w + 2] = vz[k];
      }
    }
    w++;
  }
  *n_out = std::min(w, cap);
  SF_REQUIRE(w <= cap, SF_ERR_ARG, "host arrays too small for the particle count");
  SF_API_END(ctx)
}

int sf_particles_sort(sf_ctx* ctx, int32_t sid) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_CUDA(cudaSetDevice(ctx->device));
  launch_sort(ctx, sp);
  SF_API_END(ctx)
}

int sf_particles_clear(sf_ctx* ctx, int32_t sid) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  sp->n = 0;
  sp->n_dead = 0;
  sp->cur.n = 0;
  sp->sorted = true;
  SF_API_END(ctx)
}

int sf_set_efield(sf_ctx* ctx, const double* efi, const double* efj) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && efi && efj, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaSetDevice(ctx->device));
  size_t nn = (size_t)ctx->ni * ctx->nj;
  const double* mi = static_cast<const double*>(mapped_host(efi));
  const double* mj = static_cast<const double*>(mapped_host(efj));
  if (!(mi && mj)) {
    SF_CUDA(cudaMemcpyAsync(ctx->dscratch, efi, sizeof(double) * nn, cudaMemcpyHostToDevice, ctx->stream));
    SF_CUDA(cudaMemcpyAsync(ctx->dscratch + nn, efj, sizeof(double) * nn, cudaMemcpyHostToDevice, ctx->stream));
    mi = ctx->dscratch;
    mj = ctx->dscratch + nn;
  }
  k_pack_efield<<<grid_for((int64_t)nn, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>((int)nn, mi, mj, ctx->E);
  ctx->launches++;
  SF_CUDA(cudaGetLastError());
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->efield_set = true;
  SF_API_END(ctx)
}

int sf_get_field(sf_ctx* ctx, int32_t field, int32_t sid, double* out) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && out, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaSetDevice(ctx->device));
  size_t nn = (size_t)ctx->ni * ctx->nj;
  if (field >= SF_FIELD_PHI && field <= SF_FIELD_NE) {
    int rc = sf_poisson_get_field_internal(ctx, field, out);
    if (rc != SF_OK) return rc;
    return SF_OK;
  }
  if (field == SF_FIELD_NODE_VOL) {
    std::copy(ctx->node_vol.begin(), ctx->node_vol.end(), out);
    return SF_OK;
  }
  // the fields need no particle count: a push that did not wait is read behind it on the
  // stream, with one wait at the end
  SfSpecies* sp = get_species_nowait(ctx, sid);
  switch (field) {
    case SF_FIELD_ND:
      copy_to_host(ctx, out, sp->nd, nn);
      break;
    case SF_FIELD_U:
    case SF_FIELD_V:
    case SF_FIELD_W:
      SF_REQUIRE(sp->moments_valid, SF_ERR_STATE, "moments were not deposited (SF_PUSH_MOMENTS)");
      SF_CUDA(cudaMemcpyAsync(out, sp->uvw + (field - SF_FIELD_U) * nn, sizeof(double) * nn,
                              cudaMemcpyDeviceToHost, ctx->stream));
      break;
    case SF_FIELD_NODE_VOL:
      std::copy(ctx->node_vol.begin(), ctx->node_vol.end(), out);
      break;
    case SF_FIELD_COUNT: {
      std::vector<unsigned long long> c(nn);
      SF_CUDA(cudaMemcpyAsync(c.data(), sp->count, 8 * nn, cudaMemcpyDeviceToHost, ctx->stream));
      SF_CUDA(cudaStreamSynchronize(ctx->stream));
      for (size_t u = 0; u < nn; u++) out[u] = (double)c[u] * (sp->spwt / DEP_SCALE);
      break;
    }
    default:
      SF_REQUIRE(field >= SF_FIELD_ND_AVE && field <= SF_FIELD_MPC, SF_ERR_ARG, "unknown field selector");
      SF_REQUIRE(sp->gas, SF_ERR_STATE, "no sampled moments (sf_samples_clear, SF_PUSH_SAMPLE, sf_samples_compute)");
      SF_CUDA(cudaMemcpyAsync(out, sp->gas + (size_t)(field - SF_FIELD_ND_AVE) * nn, sizeof(double) * nn,
                              cudaMemcpyDeviceToHost, ctx->stream));
  }
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  SF_API_END(ctx)
}

// Mesh.setNodeControlVolumes (core/domain/Mesh.java:1217-1296): a segment is listed on
// node (i,j) when it touches the box [i-1.01, i+1.01] x [j-1.01, j+1.01] (in cells),
// searched over the segment's bounding box grown by one node below and two above.
static bool box_touch(const double s[4], const double b1[2], const double b2[2]) {
  auto inside = [&](double x, double y) { return x >= b1[0] && x <= b2[0] && y >= b1[1] && y <= b2[1]; };
  if (inside(s[0], s[1]) || inside(s[2], s[3])) return true;
  const double f[4][4] = {{b1[0], b1[1], b2[0], b1[1]},
                          {b2[0], b1[1], b2[0], b2[1]},
                          {b2[0], b2[1], b1[0], b2[1]},
                          {b1[0], b2[1], b1[0], b1[1]}};
  for (int k = 0; k < 4; k++) {
    // parametric intersection of the segment with box edge k (LinearSegment.intersect rules)
    double x1 = s[0], y1 = s[1], x2 = s[2], y2 = s[3];
    double x3 = f[k][0], y3 = f[k][1], x4 = f[k][2], y4 = f[k][3];
    double den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
    if (den == 0) continue;
    double xp = ((x1 * y2 - y1 * x2) * (x3 - x4) - (x1 - x2) * (x3 * y4 - y3 * x4)) / den;
    double yp = ((x1 * y2 - y1 * x2) * (y3 - y4) - (y1 - y2) * (x3 * y4 - y3 * x4)) / den;
    double t0 = std::fabs(x2 - x1) > 1e-6 ? (xp - x1) / (x2 - x1) : (yp - y1) / (y2 - y1);
    if (t0 < -FLT_EPS_REF || t0 > 1 + FLT_EPS_REF) continue;
    double t1 = std::fabs(x4 - x3) > 1e-6 ? (xp - x3) / (x4 - x3) : (yp - y3) / (y4 - y3);
    if (t1 < -FLT_EPS_REF || t1 > 1 + FLT_EPS_REF) continue;
    return true;
  }
  return false;
}

int sf_build_node_segments(int32_t ni, int32_t nj, const double* x0, const double* dh, int32_t nseg,
                           const double* seg_xy, int32_t* ptr, int32_t* idx, int64_t* nnz) {
  try {
    SF_REQUIRE(ni > 0 && nj > 0 && x0 && dh && nnz && (nseg == 0 || seg_xy), SF_ERR_ARG, "bad arguments");
    std::vector<std::vector<int>> lists((size_t)ni * nj);
    for (int s = 0; s < nseg; s++) {
      const double* g = seg_xy + 4 * s;
      int lo[2], hi[2];
      for (int d = 0; d < 2; d++) {
        double mn = std::min(g[d], g[2 + d]), mx = std::max(g[d], g[2 + d]);
        lo[d] = (int)((mn - x0[d]) / dh[d]) - 1;
        hi[d] = (int)((mx - x0[d]) / dh[d]) + 2;
        lo[d] = std::max(lo[d], 0);
      }
      hi[0] = std::min(hi[0], ni - 1);
      hi[1] = std::min(hi[1], nj - 1);
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++) {
          const double b1[2] = {x0[0] + (i - 1.01) * dh[0], x0[1] + (j - 1.01) * dh[1]};
          const double b2[2] = {x0[0] + (i + 1.01) * dh[0], x0[1] + (j + 1.01) * dh[1]};
          if (!box_touch(g, b1, b2)) continue;
          auto& L = lists[(size_t)j * ni + i];
          if (std::find(L.begin(), L.end(), s) == L.end()) L.push_back(s);
        }
    }
    int64_t n = 0;
    for (size_t u = 0; u < lists.size(); u++) {
      if (ptr) ptr[u] = (int32_t)n;
      for (int s : lists[u]) {
        if (idx) idx[n] = s;
        n++;
      }
    }
    if (ptr) ptr[lists.size()] = (int32_t)n;
    *nnz = n;
    return SF_OK;
  } catch (const sf::Error& e) {
    g_create_error = e.what();
    return e.code;
  }
}

int sf_ctx_get_stream(sf_ctx* ctx, void** stream) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && stream, SF_ERR_ARG, "null argument");
  *stream = (void*)ctx->stream;
  SF_API_END(ctx)
}

int sf_timing_enable(sf_ctx* ctx, int32_t on) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null argument");
  ctx->timer.on = on != 0;
  SF_API_END(ctx)
}

int sf_timing_get(sf_ctx* ctx, const char* kernel, double* total_ms, int64_t* launches) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && kernel && total_ms && launches, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaSetDevice(ctx->device));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  timer_collect(ctx);
  *total_ms = 0;
  *launches = 0;
  for (auto& r : ctx->timer.recs)
    if (r.name == kernel) {
      *total_ms = r.ms;
      *launches = r.launches;
    }
  SF_API_END(ctx)
}

int sf_timing_reset(sf_ctx* ctx) {
  SF_API_BEGIN
  SF_REQUIRE(ctx, SF_ERR_ARG, "null argument");
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  timer_collect(ctx);
  ctx->timer.recs.clear();
  SF_API_END(ctx)
}

int sf_launch_count(sf_ctx* ctx, int64_t* launches, int32_t reset) {
  SF_API_BEGIN
  SF_REQUIRE(ctx && launches, SF_ERR_ARG, "null argument");
  *launches = ctx->launches;
  if (reset) ctx->launches = 0;
  SF_API_END(ctx)
}

int sf_get_surface_flux(sf_ctx* ctx, int32_t sid, double* flux, double* deposit) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_CUDA(cudaSetDevice(ctx->device));
  if (ctx->nseg > 0) {
    if (flux) copy_wait(flux, sp->flux, sizeof(double) * 2 * ctx->nseg, cudaMemcpyDeviceToHost, ctx->stream);
    if (deposit)
      copy_wait(deposit, sp->deposit, sizeof(double) * 2 * ctx->nseg, cudaMemcpyDeviceToHost, ctx->stream);
  }
  SF_API_END(ctx)
}

int sf_reset_surface_flux(sf_ctx* ctx, int32_t sid) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_CUDA(cudaSetDevice(ctx->device));
  int ns = std::max(ctx->nseg, 1);
  zero_wait(sp->flux, sizeof(double) * 2 * ns, ctx->stream);
  zero_wait(sp->deposit, sizeof(double) * 2 * ns, ctx->stream);
  SF_API_END(ctx)
}

}  // extern "C"
