// sf_source.cu -- particle sources sampled on the device.
//
// MaxwellianSource (sources/MaxwellianSource.java:93-125) run every step by
// SourceModule.sampleSources (core/source/SourceModule.java:231-283): particles are drawn
// uniformly along a straight boundary segment, with a drifting Maxwellian velocity from
// the reference's 12-uniform sampler (Utils.SampleMaxw3D, core/common/Utils.java:27-57,
// including its factor 1.2), rejected until v.n > 0, pushed 1e-6 dt off the surface
// (Source.sampleKinetic, core/source/Source.java:167-198) and appended with the -dt/2
// velocity rewind of KineticMaterial.addParticle (KineticMaterial.java:776-796).
// Random numbers come from counter-based Philox streams keyed by (step, particle).
#include <algorithm>
#include <cmath>

#include "sf_internal.h"

using namespace sf;

namespace {

struct InjectArgs {
  double x1, y1, x2, y2;
  double nx, ny;         // segment normal (LinearSegment: (-dy, dx)/L)
  double v_th, v_drift;  // Utils.computeVth(T, m), drift speed along the normal
  double dt;
  float qm_halfdt;       // (q/m) dt/2 for the rewind
  uint64_t seed;
  uint32_t step;
  int64_t base;          // first free slot
  int axi;               // RZ / ZR: positions uniform in the swept (frustum) area
  double r1, r2;         // radii of the segment ends
  int cold;              // UniformSource: v = normal * v_drift (no thermal spread, no dt draw)
  // null: draws outside the mesh are dropped and the others packed from `base` (counter);
  // else draw k takes slot base + k, and a draw outside the mesh leaves that slot removed
  // and is counted here
  unsigned long long* dead = nullptr;
};

// Spline.randomT on an axisymmetric mesh (core/boundaries/Spline.java:582-641) picks t so
// that the frustum area swept by [0, t] is the fraction f of the segment's area:
// t (2 r1 + t (r2 - r1)) / (r1 + r2) = f.  The reference solves it by secant steps to
// 1e-6; this is the root of the same quadratic in a cancellation-free form.
__device__ inline double frustum_t(double f, double r1, double r2) {
  const double S = r1 + r2;
  if (!(S > 0.0) || f <= 0.0) return f;
  return f * S / (r1 + sqrt(r1 * r1 + (r2 - r1) * f * S));
}


// Particle k of this step's injection on the segment of a; appended at a.base + slot.
__device__ __forceinline__ void inject_one(const MeshView& m, const ParticlesView& P, const InjectArgs& a, int64_t k,
                                           unsigned long long* counter) {
  Philox rng(a.seed, RNG_INJECT, (uint64_t)k, a.step);
  double t = rng.uniform();  // Boundary.randomT on a single segment
  if (a.axi) t = frustum_t(t, a.r1, a.r2);
  double px = a.x1 + t * (a.x2 - a.x1), py = a.y1 + t * (a.y2 - a.y1);
  double vx = 0, vy = 0, vz = 0;
  if (a.cold) {  // UniformSource.sampleParticle (sources/UniformSource.java:63-80)
    vx = a.nx * a.v_drift;
    vy = a.ny * a.v_drift;
  } else {
    // the velocity is stored in FP32: drawn in FP32 (the reference's part.dt draw, which
    // addParticle overwrites, is skipped)
    const float vt = (float)(a.v_th * 1.2), dx = (float)(a.nx * a.v_drift), dy = (float)(a.ny * a.v_drift);
    const float nx = (float)a.nx, ny = (float)a.ny;
    float fvx = 0.f, fvy = 0.f, fvz = 0.f;
    for (int tries = 0; tries < 64; tries++) {
      fvx = vt * rng.maxw1d_unit_f() + dx;
      fvy = vt * rng.maxw1d_unit_f() + dy;
      fvz = vt * rng.maxw1d_unit_f();
      if (nx * fvx + ny * fvy > 0.f) break;
    }
    vx = fvx;
    vy = fvy;
    vz = fvz;
  }
  px += vx * 1e-6 * a.dt;
  py += vy * 1e-6 * a.dt;
  double lx = (px - m.x0[0]) * m.inv_dh[0], ly = (py - m.x0[1]) * m.inv_dh[1];
  if (!(lx >= 0 && ly >= 0 && lx <= m.ni - 1 && ly <= m.nj - 1)) {  // outside every mesh
    if (a.dead) {
      P.cell[a.base + k] = DEAD;
      atomicAdd(a.dead, 1ULL);
    }
    return;
  }
  int i = (int)lx, j = (int)ly;
  if (i > m.ni - 2) i = m.ni - 2;
  if (j > m.nj - 2) j = m.nj - 2;
  const float fx = (float)(lx - i), fy = (float)(ly - j);
  const float2 eg = gather_efield(m.E, m.ni, i, j, fx, fy);
  const float ex = eg.x, ey = eg.y;
  const int64_t d = a.dead ? a.base + k : a.base + (int64_t)atomicAdd(counter, 1ULL);
  P.cell[d] = pack_cell(i, j);
  P.frac[d] = make_float2(fx, fy);
  P.vxy[d] = make_float2((float)vx - a.qm_halfdt * ex, (float)vy - a.qm_halfdt * ey);
  P.vz[d] = (float)vz;
  if (P.w) P.w[d] = 1.f;  // sources emit at the species weight
}

__global__ void k_inject_maxwellian(MeshView m, ParticlesView P, InjectArgs a, int n, unsigned long long* counter) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) inject_one(m, P, a, k, counter);
}

// ---- batched sources (one launch for all instances of a batch) -------------------
// per instance: this step's count from the flux and the remainder (Source.regenerate),
// clamped to the capacity
__global__ void k_inject_prepare(BatchDev b) {
  for (int i = threadIdx.x; i < b.n; i += blockDim.x) {
    const BatchInst& I = b.insts[i];
    const int64_t base = b.n_dev[i];
    int64_t num = 0;
    if (I.src_on) {
      const double mp = I.mp_step + b.rem_dev[i];
      num = (int64_t)mp;
      b.rem_dev[i] = mp - (double)num;
      if (base + num > I.cap) {
        num = I.cap > base ? I.cap - base : 0;
        atomicExch(b.overflow, 1);
      }
    }
    b.num_dev[i] = num;
    b.base_dev[i] = base;
    b.added_dev[i] = 0ULL;
  }
}

__global__ void k_inject_batch(BatchDev b) {
  const int i = blockIdx.y;
  const BatchInst& I = b.insts[i];
  const int64_t num = b.num_dev[i];
  if (num <= 0) return;
  InjectArgs a;
  a.x1 = I.sx1;
  a.y1 = I.sy1;
  a.x2 = I.sx2;
  a.y2 = I.sy2;
  a.nx = I.snx;
  a.ny = I.sny;
  a.v_th = I.v_th;
  a.v_drift = I.v_drift;
  a.dt = I.src_dt;
  a.qm_halfdt = I.qm_halfdt;
  a.seed = I.src_seed;
  a.step = *b.step_dev;
  a.base = b.base_dev[i];
  a.axi = 0;
  a.r1 = a.r2 = 0.0;
  a.cold = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < num; k += (int64_t)gridDim.x * blockDim.x)
    inject_one(I.m, I.P, a, k, &b.added_dev[i]);
}

}  // namespace

namespace sf {
void batch_inject(const BatchDev& b, cudaStream_t stream, int num_sms) {
  k_inject_prepare<<<1, 256, 0, stream>>>(b);
  k_inject_batch<<<dim3(std::max(1, num_sms / 8), b.n), 256, 0, stream>>>(b);
  SF_CUDA(cudaGetLastError());
}
}  // namespace sf

namespace {

// Spline.isOnLine (core/boundaries/Spline.java:833-862) for a straight segment
__device__ bool seg_on_line(const Seg4 s, double x, double y) {
  double t;
  if (s.z != s.x) {
    t = (x - s.x) / (s.z - s.x);
    if (t < -FLT_EPS_REF || t > 1.0 + FLT_EPS_REF) return false;
  } else {
    t = (y - s.y) / (s.w - s.y);
    if (t < -FLT_EPS_REF || t > 1.0 + FLT_EPS_REF) return false;
  }
  const double d1 = s.x + t * (s.z - s.x) - x, d2 = s.y + t * (s.w - s.y) - y;
  const double l2 = (s.z - s.x) * (s.z - s.x) + (s.w - s.y) * (s.w - s.y);
  return !((d1 * d1 + d2 * d2) / l2 > FLT_EPS_REF);
}

// BoundaryModule.isInternal (core/boundaries/BoundaryModule.java:245-251) with
// Spline.visibleSegment (Spline.java:881-929) and Spline.isInternal (:806-830) for
// straight segments: the first non-virtual, non-open segment whose midpoint (closestPos
// of a linear segment is 1/2) is seen from (x, y) without crossing another such
// segment, or on which the point lies, decides: internal when the point is on it or
// behind its normal (-dy, dx) / L.
__device__ bool point_internal(const MeshView& m, double x, double y) {
  const double xp[2] = {x, y};
  for (int s = 0; s < m.nseg; s++) {
    const int bt = m.seg_btype[s];
    if (bt == SF_BT_VIRTUAL || bt == SF_BT_OPEN) continue;
    const Seg4 g = m.seg_xy[s];
    if (seg_on_line(g, x, y)) return true;
    const double xc[2] = {0.5 * (g.x + g.z), 0.5 * (g.y + g.w)};
    bool blocked = false;
    for (int s2 = 0; s2 < m.nseg && !blocked; s2++) {
      if (s2 == s) continue;
      const int bt2 = m.seg_btype[s2];
      if (bt2 == SF_BT_VIRTUAL || bt2 == SF_BT_OPEN) continue;
      double t[2];
      seg_intersect(m.seg_xy[s2], xp, xc, t);
      blocked = t[0] >= 0;
    }
    if (blocked) continue;
    const double dx = g.z - g.x, dy = g.w - g.y, len = sqrt(dx * dx + dy * dy);
    const double rx = x - xc[0], ry = y - xc[1];
    const double cs = (rx * (-dy / len) + ry * (dx / len)) / sqrt(rx * rx + ry * ry);
    return cs <= 0;
  }
  return false;
}

struct PreloadArgs {
  double v_th;        // Utils.computeVth(max(T, 50 K), m)
  double dt;
  float qm_halfdt;
  uint64_t seed;
  uint32_t step;
  int64_t base;       // first slot
};

// VolumeSource.sampleParticle (core/source/VolumeSource.java:63-119) for every cell c:
// particles start[c] .. start[c + 1] of this call, uniform in the cell's logical square,
// Maxwellian (Utils.SampleMaxw3D, its factor 1.2 included); internal ones are not added
// (their slots are left removed); then Source.sampleKinetic's 1e-6 dt push off and the
// -dt/2 rewind of KineticMaterial.addParticle.
__global__ void k_preload(MeshView m, ParticlesView P, PreloadArgs a, const int64_t* __restrict__ start, int ncx,
                          int ncells, unsigned long long* n_internal) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
    const int ci = c % ncx, cj = c / ncx;
    for (int64_t k = start[c]; k < start[c + 1]; k++) {
      Philox rng(a.seed, RNG_INJECT, (uint64_t)k, a.step);
      const double li = ci + rng.uniform(), lj = cj + rng.uniform();
      double px = m.x0[0] + li * m.dh[0], py = m.x0[1] + lj * m.dh[1];
      const double vx = (a.v_th * 1.2) * rng.maxw1d_unit();
      const double vy = (a.v_th * 1.2) * rng.maxw1d_unit();
      const double vz = (a.v_th * 1.2) * rng.maxw1d_unit();
      const int64_t d = a.base + k;
      if (point_internal(m, px, py)) {
        P.cell[d] = DEAD;
        if (P.w) P.w[d] = 1.f;
        atomicAdd(n_internal, 1ULL);
        continue;
      }
      px += vx * 1e-6 * a.dt;
      py += vy * 1e-6 * a.dt;
      double lx = (px - m.x0[0]) * m.inv_dh[0], ly = (py - m.x0[1]) * m.inv_dh[1];
      lx = fmin(fmax(lx, 0.0), m.ni - 1.0);
      ly = fmin(fmax(ly, 0.0), m.nj - 1.0);
      int i = (int)lx, j = (int)ly;
      if (i > m.ni - 2) i = m.ni - 2;
      if (j > m.nj - 2) j = m.nj - 2;
      const float fx = (float)(lx - i), fy = (float)(ly - j);
      const float2 eg = gather_efield(m.E, m.ni, i, j, fx, fy);
      const float ex = eg.x, ey = eg.y;
      P.cell[d] = pack_cell(i, j);
      P.frac[d] = make_float2(fx, fy);
      P.vxy[d] = make_float2((float)vx - a.qm_halfdt * ex, (float)vy - a.qm_halfdt * ey);
      P.vz[d] = (float)vz;
      if (P.w) P.w[d] = 1.f;
    }
  }
}

// One segment source of num particles (MaxwellianSource or, cold, UniformSource)
// wait = false: every draw takes its own slot and the host reads nothing back (a draw that
// lands outside the mesh leaves its slot removed, counted with the pushes' removals)
int64_t segment_source(sf_ctx* ctx, SfSpecies* sp, int32_t sid, const double* seg, int64_t num, double v_drift,
                       double temp, double dt, int cold, bool wait = true) {
  const double dx = seg[2] - seg[0], dy = seg[3] - seg[1];
  const double len = std::sqrt(dx * dx + dy * dy);
  SF_REQUIRE(sp->n + num <= sp->cap, SF_ERR_OOM, "species capacity exceeded by the source");
  InjectArgs a;
  a.x1 = seg[0];
  a.y1 = seg[1];
  a.x2 = seg[2];
  a.y2 = seg[3];
  a.nx = -dy / len;
  a.ny = dx / len;
  a.v_th = std::sqrt(2 * KB * temp / sp->mass);
  a.v_drift = v_drift;
  a.dt = dt;
  a.qm_halfdt = (float)(sp->charge / sp->mass * 0.5 * dt);
  a.seed = ctx->seed ^ (0x9E3779B97F4A7C15ULL * (uint64_t)(sid + 1));
  a.step = ctx->rng_epoch++;
  a.base = sp->n;
  a.axi = ctx->domain != SF_DOMAIN_XY;
  a.r1 = ctx->domain == SF_DOMAIN_RZ ? seg[0] : seg[1];
  a.r2 = ctx->domain == SF_DOMAIN_RZ ? seg[2] : seg[3];
  a.cold = cold;
  unsigned long long* cnt = ctx->counters + 7;
  if (!wait) {
    a.dead = sp->acc;  // acc[0]: removed slots the host has not read yet
    k_inject_maxwellian<<<(int)((num + 255) / 256), 256, 0, ctx->stream>>>(ctx->mesh_view(), sp->cur, a, (int)num,
                                                                          cnt);
    ctx->launches++;
    SF_CUDA(cudaGetLastError());
    sp->acc_pending = true;
    sp->n += num;
    sp->cur.n = sp->n;
    sp->sorted = false;
    return num;
  }
  SF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream));
  k_inject_maxwellian<<<(int)((num + 255) / 256), 256, 0, ctx->stream>>>(ctx->mesh_view(), sp->cur, a, (int)num, cnt);
  ctx->launches++;
  SF_CUDA(cudaGetLastError());
  unsigned long long added = 0;
  SF_CUDA(cudaMemcpyAsync(&added, cnt, sizeof(added), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  sp->n += (int64_t)added;
  sp->cur.n = sp->n;
  sp->sorted = false;
  return (int64_t)added;
}

double segment_length(const double* seg) {
  const double dx = seg[2] - seg[0], dy = seg[3] - seg[1];
  return std::sqrt(dx * dx + dy * dy);
}

}  // namespace

extern "C" int sf_source_maxwellian(sf_ctx* ctx, int32_t sid, const double* seg, double den, double v_drift,
                                    double temp, double dt, double* rem, int64_t* n_added) {
  SF_API_BEGIN
  // without n_added nothing is read back: the slot count is all the source needs
  SfSpecies* sp = n_added ? get_species(ctx, sid) : get_species_nowait(ctx, sid);
  SF_REQUIRE(seg && rem, SF_ERR_ARG, "null argument");
  SF_REQUIRE(den >= 0 && temp >= 0 && dt > 0, SF_ERR_ARG, "bad source parameters");
  SF_REQUIRE(ctx->efield_set, SF_ERR_STATE, "electric field not set (the rewind gathers E)");
  SF_CUDA(cudaSetDevice(ctx->device));
  const double len = segment_length(seg);
  SF_REQUIRE(len > 0, SF_ERR_ARG, "degenerate source segment");
  // MaxwellianSource ctor (MaxwellianSource.java:60-80): mdot from den; Source.regenerate
  const double v_mean = std::sqrt(8 * KB * temp / (PI * sp->mass));
  // LinearSegment.area (core/boundaries/LinearSegment.java:51-76): length x 1 m in XY, the
  // lateral area of the swept conical frustum pi (r1 + r2) L in RZ / ZR
  double area = len;
  if (ctx->domain == SF_DOMAIN_ZR) area = PI * (seg[1] + seg[3]) * len;
  if (ctx->domain == SF_DOMAIN_RZ) area = PI * (seg[0] + seg[2]) * len;
  const double mdot = den * area * (v_drift + v_mean / 4) * sp->mass;
  const double mp = (mdot * dt) / (sp->mass * sp->spwt) + *rem;
  const int64_t num = (int64_t)mp;
  *rem = mp - (double)num;
  if (n_added) *n_added = 0;
  if (num <= 0) return SF_OK;
  const int64_t added = segment_source(ctx, sp, sid, seg, num, v_drift, temp, dt, 0, n_added != nullptr);
  if (n_added) *n_added = added;
  SF_API_END(ctx)
}

extern "C" int sf_source_uniform(sf_ctx* ctx, int32_t sid, const double* seg, double mdot, double v_drift, double dt,
                                 double* rem, int64_t* n_added) {
  SF_API_BEGIN
  SfSpecies* sp = n_added ? get_species(ctx, sid) : get_species_nowait(ctx, sid);
  SF_REQUIRE(seg && rem, SF_ERR_ARG, "null argument");
  SF_REQUIRE(mdot >= 0 && dt > 0, SF_ERR_ARG, "bad source parameters");
  SF_REQUIRE(ctx->efield_set, SF_ERR_STATE, "electric field not set (the rewind gathers E)");
  SF_CUDA(cudaSetDevice(ctx->device));
  SF_REQUIRE(segment_length(seg) > 0, SF_ERR_ARG, "degenerate source segment");
  // Source.regenerate (core/source/Source.java:123-134) with the given mass flow rate
  const double mp = (mdot * dt) / (sp->mass * sp->spwt) + *rem;
  const int64_t num = (int64_t)mp;
  *rem = mp - (double)num;
  if (n_added) *n_added = 0;
  if (num <= 0) return SF_OK;
  const int64_t added = segment_source(ctx, sp, sid, seg, num, v_drift, 0.0, dt, 1, n_added != nullptr);
  if (n_added) *n_added = added;
  SF_API_END(ctx)
}

extern "C" int sf_source_preload(sf_ctx* ctx, int32_t sid, double den, double temp, double dt, int64_t* n_added) {
  SF_API_BEGIN
  SfSpecies* sp = get_species(ctx, sid);
  SF_REQUIRE(n_added && den >= 0 && temp >= 0 && dt > 0, SF_ERR_ARG, "bad preload parameters");
  SF_REQUIRE(ctx->efield_set, SF_ERR_STATE, "electric field not set (the rewind gathers E)");
  SF_CUDA(cudaSetDevice(ctx->device));
  // VolumePreloadSource.regenerate (sources/VolumePreloadSource.java:44-66) sets dn = den
  // and T = temp; VolumeSource.findNextCell / sampleParticle (core/source/VolumeSource.java:
  // 63-170) then make, per cell, particles while the remaining number num_rem =
  // dn cellVol > spwt, each taking spwt: ceil(num_rem / spwt) - 1 of them.
  const int ncx = ctx->ni - 1, ncy = ctx->nj - 1, nc = ncx * ncy;
  std::vector<int64_t> start(nc + 1, 0);
  for (int j = 0; j < ncy; j++)
    for (int i = 0; i < ncx; i++) {
      // Mesh.cellVol = nodeVol(i + 1/2, j + 1/2) (core/domain/Mesh.java:1038-1040)
      double v = ctx->dh[0] * ctx->dh[1];
      if (ctx->domain == SF_DOMAIN_RZ) v *= 2 * PI * (ctx->x0[0] + (i + 0.5) * ctx->dh[0]);
      if (ctx->domain == SF_DOMAIN_ZR) v *= 2 * PI * (ctx->x0[1] + (j + 0.5) * ctx->dh[1]);
      const double r = den * v / sp->spwt;
      const int64_t k = r > 1.0 ? (int64_t)std::ceil(r) - 1 : 0;
      start[(size_t)j * ncx + i + 1] = k;
    }
  for (int c = 0; c < nc; c++) start[c + 1] += start[c];
  const int64_t num = start[nc];
  *n_added = 0;
  if (num == 0) return SF_OK;
  SF_REQUIRE(sp->n + num <= sp->cap, SF_ERR_OOM, "species capacity exceeded by the preload");
  // the cell prefix in the context's FP64 scratch (2 * ni * nj doubles >= nc + 1 int64)
  int64_t* d_start = reinterpret_cast<int64_t*>(ctx->dscratch);
  copy_wait(d_start, start.data(), sizeof(int64_t) * (nc + 1), cudaMemcpyHostToDevice, ctx->stream);
  PreloadArgs a;
  a.v_th = std::sqrt(2 * KB * std::max(temp, 50.0) / sp->mass);
  a.dt = dt;
  a.qm_halfdt = (float)(sp->charge / sp->mass * 0.5 * dt);
  a.seed = ctx->seed ^ (0xA5A5A5A5ULL * (uint64_t)(sid + 1));
  a.step = ctx->rng_epoch++;
  a.base = sp->n;
  unsigned long long* cnt = ctx->counters + 7;
  SF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream));
  k_preload<<<grid_for(nc, 128, ctx->num_sms * 8), 128, 0, ctx->stream>>>(ctx->mesh_view(), sp->cur, a, d_start, ncx,
                                                                          nc, cnt);
  ctx->launches++;
  SF_CUDA(cudaGetLastError());
  unsigned long long internal = 0;
  SF_CUDA(cudaMemcpyAsync(&internal, cnt, sizeof(internal), cudaMemcpyDeviceToHost, ctx->stream));
  SF_CUDA(cudaStreamSynchronize(ctx->stream));
  sp->n += num;
  sp->cur.n = sp->n;
  sp->n_dead += (int64_t)internal;
  sp->sorted = false;
  *n_added = num - (int64_t)internal;
  SF_API_END(ctx)
}
