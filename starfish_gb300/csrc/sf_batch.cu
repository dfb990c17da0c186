// sf_batch.cu -- many independent ES-PIC instances advanced together.
//
// A batch holds contexts of different mesh sizes and particle counts (each a complete
// Starfish case: mesh, one kinetic species, Poisson-Boltzmann solver).  One step of all
// instances is
//   1. device phase, one CUDA graph on the batch stream, no host values: the batched
//      Maxwellian sources (counts and remainders on the device), one push launch over
//      the tiles of every instance (a device prefix of the per-instance tile counts),
//      one launch of the exact surface path over the slow queues of all instances cut
//      into equal chunks (a device prefix of the chunk counts, so one long queue is
//      spread over the whole GPU), and the per-instance densities;
//   2. field phase: per instance rho, the nonlinear Poisson solve and E on the
//      instance's own stream, issued by a pool of host threads so that the solves of
//      different instances overlap on the GPU (each solve's Newton steps are CUDA graphs
//      with one residual check on the host per step).
// Every sort_interval steps the instances are cell-sorted (per instance, between steps).
// An autotuner picks the launch shape (push blocks per SM, exact-path blocks per SM) by
// timing the device phase, and the inner PCG iterations per Newton step per
// mesh-size bucket by timing the solves, during the first steps.
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sf_internal.h"

using namespace sf;

namespace {

// persistent pool: run(f) calls f(w) on workers w = 0..n-1 and waits for all of them
class Pool {
 public:
  explicit Pool(int n) : n_(n) {
    for (int w = 0; w < n; w++) th_.emplace_back([this, w] { loop(w); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(m_);
      quit_ = true;
      gen_++;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void run(const std::function<void(int)>& f) {
    std::unique_lock<std::mutex> g(m_);
    job_ = &f;
    pending_ = n_;
    gen_++;
    cv_.notify_all();
    done_.wait(g, [this] { return pending_ == 0; });
    job_ = nullptr;
  }
  int size() const { return n_; }

 private:
  void loop(int w) {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(int)>* f;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return gen_ != seen; });
        seen = gen_;
        if (quit_) return;
        f = job_;
      }
      (*f)(w);
      {
        std::lock_guard<std::mutex> g(m_);
        if (--pending_ == 0) done_.notify_one();
      }
    }
  }
  int n_;
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int pending_ = 0;
  uint64_t gen_ = 0;
  bool quit_ = false;
};

constexpr int N_BUCKETS = 3;           // mesh nodes < 4096, < 16384, larger
constexpr int CYCLE_CHOICES[3] = {2, 3, 4};
constexpr int SHAPES[4][2] = {{4, 16}, {2, 16}, {1, 16}, {4, 8}};  // push blocks per SM, slow-path blocks per SM
constexpr int TRIAL_STEPS = 2;         // steps timed per candidate

int bucket_of(const sf_ctx* c) {
  const int nn = c->ni * c->nj;
  return nn < 4096 ? 0 : (nn < 16384 ? 1 : 2);
}

}  // namespace

struct sf_batch {
  int device = 0;
  int n = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_dev = nullptr, ev0 = nullptr, ev1 = nullptr;
  std::vector<sf_ctx*> ctx;
  std::vector<int> sid;
  std::vector<BatchInst> h;
  BatchDev d{};
  std::vector<void*> allocs;
  double dt = 0;
  bool table_ready = false;
  bool dirty = true;  // the instance table must be rebuilt before the next step
  int64_t steps = 0;
  int sort_interval = 16;
  // graphs of the device phase, one per push launch shape
  cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
  // autotuner
  int shape = -1;                     // chosen push launch shape (index into SHAPES)
  double shape_ms[4] = {0, 0, 0, 0};
  int shape_n[4] = {0, 0, 0, 0};
  int cycles[N_BUCKETS] = {-1, -1, -1};
  double cyc_ms[N_BUCKETS][3] = {};
  int cyc_n[N_BUCKETS][3] = {};
  std::unique_ptr<Pool> pool;
  sf::BatchPoisson* bp = nullptr;  // batched field phase (created at the first step that uses it)
  std::string err;
  // source parameters per instance (den, v_drift, temp, seg) for the step's dt
  struct Src {
    bool on = false;
    double seg[4] = {0, 0, 0, 0};
    double den = 0, v_drift = 0, temp = 0;
  };
  std::vector<Src> src;
};

namespace {

template <typename T>
T* balloc(sf_batch* b, size_t count) {
  void* p = nullptr;
  SF_CUDA(cudaMalloc(&p, std::max<size_t>(sizeof(T) * count, 16)));
  zero_wait(p, std::max<size_t>(sizeof(T) * count, 16), b->stream);
  b->allocs.push_back(p);
  return static_cast<T*>(p);
}

// host view of one instance for the batched kernels (dt-dependent push arguments)
BatchInst make_inst(sf_batch* b, int i) {
  sf_ctx* c = b->ctx[i];
  SfSpecies* sp = get_species(c, b->sid[i]);
  BatchInst I{};
  I.m = c->mesh_view();
  I.P = sp->cur;
  const double dt = b->dt;
  PushArgs& a = I.a;
  a.qm_dt = (float)(sp->charge / sp->mass * dt);
  a.dt_dx = (float)(dt / c->dh[0]);
  a.dt_dy = (float)(dt / c->dh[1]);
  a.dt = (float)dt;
  a.dx = (float)c->dh[0];
  a.dy = (float)c->dh[1];
  a.r0x = (float)c->x0[0];
  a.r0y = (float)c->x0[1];
  a.dt64 = dt;
  a.qm = sp->charge / sp->mass;
  a.charge = sp->charge;
  a.spwt = sp->spwt;
  a.seed = c->seed;
  a.step = sp->step;
  I.sa.sv.model = sp->seg_model;
  I.sa.sv.param = sp->seg_param;
  I.sa.sv.flux = sp->flux;
  I.sa.sv.deposit = sp->deposit;
  I.sa.counters = c->counters;
  I.sa.stats_slow = c->stats_partial + (size_t)8 * (c->stats_blocks - 1);
  I.sa.stats = 0;  // the batch reports no push totals
  I.sa.sv.product = nullptr;  // surface products are per context (sf_push_deposit)
  I.sa.sv.prod = nullptr;
  I.count = sp->count;
  I.slow_idx = c->slow_idx;
  I.nd = sp->nd;
  I.nd_factor = sp->nd_factor;
  I.nd_back = sp->nd_back;
  I.cap = sp->cap;
  const sf_batch::Src& s = b->src[i];
  I.src_on = s.on ? 1 : 0;
  if (s.on) {
    // MaxwellianSource flux on a straight XY segment (MaxwellianSource.java:60-125,
    // LinearSegment.area: length x 1 m)
    const double dx = s.seg[2] - s.seg[0], dy = s.seg[3] - s.seg[1];
    const double len = std::sqrt(dx * dx + dy * dy);
    const double v_mean = std::sqrt(8 * KB * s.temp / (PI * sp->mass));
    const double mdot = s.den * len * (s.v_drift + v_mean / 4) * sp->mass;
    I.sx1 = s.seg[0];
    I.sy1 = s.seg[1];
    I.sx2 = s.seg[2];
    I.sy2 = s.seg[3];
    I.snx = -dy / len;
    I.sny = dx / len;
    I.v_th = std::sqrt(2 * KB * s.temp / sp->mass);
    I.v_drift = s.v_drift;
    I.src_dt = dt;
    I.mp_step = (mdot * dt) / (sp->mass * sp->spwt);
    I.qm_halfdt = (float)(sp->charge / sp->mass * 0.5 * dt);
    I.src_seed = c->seed ^ (0x9E3779B97F4A7C15ULL * (uint64_t)(b->sid[i] + 1));
  }
  return I;
}

// host particle bookkeeping from the device counts
void pull_counts(sf_batch* b) {
  std::vector<int64_t> n(b->n), dead(b->n);
  SF_CUDA(cudaMemcpyAsync(n.data(), b->d.n_dev, 8 * (size_t)b->n, cudaMemcpyDeviceToHost, b->stream));
  SF_CUDA(cudaMemcpyAsync(dead.data(), b->d.dead_dev, 8 * (size_t)b->n, cudaMemcpyDeviceToHost, b->stream));
  SF_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->n; i++) {
    SfSpecies* sp = get_species(b->ctx[i], b->sid[i]);
    sp->n = n[i];
    sp->cur.n = n[i];
    sp->n_dead = dead[i];
    sp->sorted = false;
  }
}

// device counts and instance table from the host state (after a sort or a change of dt);
// the device-advanced push steps are kept
void push_table(sf_batch* b) {
  std::vector<int64_t> n(b->n), dead(b->n);
  if (b->table_ready) {
    std::vector<BatchInst> cur(b->n);
    copy_wait(cur.data(), b->d.insts, sizeof(BatchInst) * b->n, cudaMemcpyDeviceToHost, b->stream);
    for (int i = 0; i < b->n; i++) get_species(b->ctx[i], b->sid[i])->step = cur[i].a.step;
  }
  for (int i = 0; i < b->n; i++) {
    b->h[i] = make_inst(b, i);
    SfSpecies* sp = get_species(b->ctx[i], b->sid[i]);
    n[i] = sp->n;
    dead[i] = sp->n_dead;
  }
  copy_wait(b->d.insts, b->h.data(), sizeof(BatchInst) * b->n, cudaMemcpyHostToDevice, b->stream);
  copy_wait(b->d.n_dev, n.data(), 8 * (size_t)b->n, cudaMemcpyHostToDevice, b->stream);
  copy_wait(b->d.dead_dev, dead.data(), 8 * (size_t)b->n, cudaMemcpyHostToDevice, b->stream);
  b->table_ready = true;
}

void device_phase(sf_batch* b, int shape, cudaStream_t s) {
  batch_inject(b->d, s, b->num_sms);
  batch_push(b->d, s, b->num_sms, SHAPES[shape][0], SHAPES[shape][1]);
}

cudaGraphExec_t graph_for(sf_batch* b, int shape) {
  if (b->graph[shape]) return b->graph[shape];
  cudaGraph_t g = nullptr;
  SF_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  try {
    device_phase(b, shape, b->stream);
  } catch (...) {
    cudaStreamEndCapture(b->stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  SF_CUDA(cudaStreamEndCapture(b->stream, &g));
  const cudaError_t e = cudaGraphInstantiate(&b->graph[shape], g, 0);
  cudaGraphDestroy(g);
  SF_CUDA(e);
  return b->graph[shape];
}

int pick_best(const double* ms, const int* cnt, int k) {
  int best = 0;
  for (int c = 1; c < k; c++)
    if (cnt[c] > 0 && (cnt[best] == 0 || ms[c] / cnt[c] < ms[best] / cnt[best])) best = c;
  return best;
}

}  // namespace

extern "C" {

int sf_batch_create(sf_ctx** ctxs, const int32_t* sids, int32_t n, int32_t threads, sf_batch** out) {
  sf_batch* b = nullptr;
  try {
    SF_REQUIRE(ctxs && sids && out && n > 0, SF_ERR_ARG, "null argument or empty batch");
    b = new sf_batch();
    b->n = n;
    b->device = ctxs[0]->device;
    for (int i = 0; i < n; i++) {
      SF_REQUIRE(ctxs[i], SF_ERR_ARG, "null context in the batch");
      SF_REQUIRE(ctxs[i]->device == b->device, SF_ERR_ARG, "all instances of a batch must be on one device");
      SF_REQUIRE(ctxs[i]->domain == SF_DOMAIN_XY, SF_ERR_ARG, "batched instances must be XY meshes");
      for (int k = 0; k < i; k++) SF_REQUIRE(ctxs[k] != ctxs[i], SF_ERR_ARG, "a context appears twice in the batch");
      b->ctx.push_back(ctxs[i]);
      b->sid.push_back(sids[i]);
    }
    SF_CUDA(cudaSetDevice(b->device));
    b->num_sms = ctxs[0]->num_sms;
    SF_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    SF_CUDA(cudaEventCreateWithFlags(&b->ev_dev, cudaEventDisableTiming));
    SF_CUDA(cudaEventCreate(&b->ev0));
    SF_CUDA(cudaEventCreate(&b->ev1));
    b->h.resize(n);
    b->src.resize(n);
    b->d.n = n;
    b->d.insts = balloc<BatchInst>(b, n);
    b->d.n_dev = balloc<int64_t>(b, n);
    b->d.dead_dev = balloc<int64_t>(b, n);
    b->d.rem_dev = balloc<double>(b, n);
    b->d.num_dev = balloc<int64_t>(b, n);
    b->d.base_dev = balloc<int64_t>(b, n);
    b->d.added_dev = balloc<unsigned long long>(b, n);
    b->d.tile_start = balloc<int64_t>(b, n + 1);
    b->d.chunk_start = balloc<int64_t>(b, n + 1);
    b->d.step_dev = balloc<uint32_t>(b, 1);
    b->d.overflow = balloc<int>(b, 1);
    b->d.any_weighted = 0;
    for (int i = 0; i < n; i++) b->d.any_weighted |= get_species(ctxs[i], sids[i])->weighted ? 1 : 0;
    b->pool.reset(new Pool(std::max(1, std::min<int>(threads > 0 ? threads : 8, n))));
    *out = b;
    return SF_OK;
  } catch (const sf::Error& e) {
    if (b) {
      for (void* p : b->allocs) cudaFree(p);
      delete b;
    }
    return e.code;
  }
}

int sf_batch_destroy(sf_batch* b) {
  if (!b) return SF_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  // the contexts go on from where the batch left them: their push steps (surface RNG
  // epochs) were advanced on the device (the particle counts already follow every step)
  if (b->table_ready) {
    std::vector<BatchInst> cur(b->n);
    if (cudaMemcpyAsync(cur.data(), b->d.insts, sizeof(BatchInst) * b->n, cudaMemcpyDeviceToHost, b->stream) ==
            cudaSuccess &&
        cudaStreamSynchronize(b->stream) == cudaSuccess)
      for (int i = 0; i < b->n; i++) b->ctx[i]->species[b->sid[i]]->step = cur[i].a.step;  // checked at create
  }
  for (auto& g : b->graph)
    if (g) cudaGraphExecDestroy(g);
  sf::batch_poisson_destroy(b->bp);
  b->bp = nullptr;
  for (void* p : b->allocs) cudaFree(p);
  if (b->ev_dev) cudaEventDestroy(b->ev_dev);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  b->pool.reset();
  delete b;
  return SF_OK;
}

const char* sf_batch_last_error(const sf_batch* b) { return b ? b->err.c_str() : ""; }

int sf_batch_set_source(sf_batch* b, int32_t i, const double* seg, double den, double v_drift, double temp) {
  try {
    SF_REQUIRE(b && i >= 0 && i < b->n && seg, SF_ERR_ARG, "bad instance or null segment");
    SF_REQUIRE(den >= 0 && temp >= 0, SF_ERR_ARG, "bad source parameters");
    const double dx = seg[2] - seg[0], dy = seg[3] - seg[1];
    SF_REQUIRE(dx * dx + dy * dy > 0, SF_ERR_ARG, "degenerate source segment");
    sf_batch::Src& s = b->src[i];
    s.on = true;
    std::memcpy(s.seg, seg, sizeof(s.seg));
    s.den = den;
    s.v_drift = v_drift;
    s.temp = temp;
    b->dirty = true;  // the instance table is rebuilt at the next step
    for (auto& g : b->graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    return SF_OK;
  } catch (const sf::Error& e) {
    if (b) b->err = e.what();
    return e.code;
  }
}

int sf_batch_step(sf_batch* b, double dt, const sf_poisson_params* prm, sf_batch_stats* st) {
  try {
    SF_REQUIRE(b && prm && dt > 0, SF_ERR_ARG, "null argument or bad dt");
    SF_CUDA(cudaSetDevice(b->device));
    int aw = 0;
    for (int i = 0; i < b->n; i++) {
      SF_REQUIRE(b->ctx[i]->efield_set, SF_ERR_STATE, "an instance has no electric field (solve or set E first)");
      aw |= get_species(b->ctx[i], b->sid[i])->weighted ? 1 : 0;
    }
    if (aw != b->d.any_weighted) {
      // a species was switched to per-particle weights since the graphs were captured
      b->d.any_weighted = aw;
      for (auto& g : b->graph)
        if (g) {
          cudaGraphExecDestroy(g);
          g = nullptr;
        }
    }
    std::string errs;
    std::mutex em;
    auto fail = [&](int i, const std::string& what) {
      std::lock_guard<std::mutex> g(em);
      if (errs.empty()) errs = "instance " + std::to_string(i) + ": " + what;
    };
    // cell sort of every instance (its first step, then every sort_interval steps)
    const bool sort_now = b->steps % b->sort_interval == 0;
    if (sort_now || b->dirty || dt != b->dt) {
      if (b->table_ready) pull_counts(b);
      if (dt != b->dt) {
        b->dt = dt;
        for (auto& g : b->graph)
          if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
          }
      }
      if (sort_now) {
        const int T = b->pool->size();
        b->pool->run([&](int w) {
          for (int i = w; i < b->n; i += T) {
            try {
              SF_CUDA(cudaSetDevice(b->device));
              // keys half a sort interval ahead, as the single-context automatic sort
              sf_ctx* c = b->ctx[i];
              const double tau = 0.5 * b->sort_interval * dt;
              SfSpecies* si = get_species(c, b->sid[i]);
              launch_sort(c, si, (float)(tau / c->dh[0]), (float)(tau / c->dh[1]), si->sort_qb);
            } catch (const std::exception& e) {
              fail(i, e.what());
            }
          }
        });
        SF_REQUIRE(errs.empty(), SF_ERR_CUDA, errs);
      }
      push_table(b);
      b->dirty = false;
    }
    // push launch shape: tuning trials first, then the fastest
    int shape = b->shape;
    const bool tuning_shape = shape < 0;
    if (tuning_shape) shape = (int)((b->steps / TRIAL_STEPS) % 4);
    // the device phase needs the previous step's fields (the pool has joined)
    SF_CUDA(cudaEventRecord(b->ev0, b->stream));
    SF_CUDA(cudaGraphLaunch(graph_for(b, shape), b->stream));
    SF_CUDA(cudaEventRecord(b->ev1, b->stream));
    SF_CUDA(cudaEventRecord(b->ev_dev, b->stream));
    // field phase: rho, Poisson, E of every instance
    const int tuning_step = (int)(b->steps % (3 * TRIAL_STEPS)) / TRIAL_STEPS;  // cycles choice under trial
    std::vector<double> solve_ms(b->n, 0.0);
    std::vector<int> newton(b->n, 0);
    double field_sum = 0, field_max = 0;
    if (!prm->use_learned) {
      // one launch per stage for all instances on the batch stream (after the device phase)
      if (!b->bp) b->bp = batch_poisson_create(b->ctx.data(), b->n, b->num_sms, b->stream);
      std::vector<int> iters(b->n), status(b->n);
      std::vector<sf_solve_stats> ss(b->n);
      for (int i = 0; i < b->n; i++) {
        const int bk = bucket_of(b->ctx[i]);
        iters[i] = b->cycles[bk] > 0 ? b->cycles[bk] : CYCLE_CHOICES[tuning_step];
      }
      const float ms = batch_poisson_step(b->bp, *prm, iters.data(), ss.data(), status.data());
      field_sum = field_max = ms;
      for (int i = 0; i < b->n; i++) {
        solve_ms[i] = ms;  // one time for all: the tuner then picks one PCG count for every bucket
        newton[i] = ss[i].newton_it;
      }
      for (int i = 0; i < b->n; i++)
        if (status[i] != 1)
          SF_REQUIRE(false, status[i] == 3 ? SF_ERR_DIVERGED : SF_ERR_NOT_CONVERGED,
                     "instance " + std::to_string(i) +
                         (status[i] == 3 ? ": Solver diverged (non-finite residual)"
                                         : ": Poisson solve did not reach the residual tolerance"));
    } else {
    // the learned warm start is per context: the instances' own solves on their streams,
    // issued by the host thread pool
    const int T = b->pool->size();
    b->pool->run([&](int w) {
      for (int i = w; i < b->n; i += T) {
        try {
          sf_ctx* c = b->ctx[i];
          SF_CUDA(cudaSetDevice(b->device));
          SF_CUDA(cudaStreamWaitEvent(c->stream, b->ev_dev, 0));
          int rc = sf_update_rho(c);
          SF_REQUIRE(rc == SF_OK, rc, sf_last_error(c));
          sf_poisson_params p = *prm;
          const int bk = bucket_of(c);
          p.cycles = b->cycles[bk] > 0 ? b->cycles[bk] : CYCLE_CHOICES[tuning_step];
          sf_solve_stats ss{};
          rc = sf_poisson_nl(c, &p, nullptr, nullptr, &ss);
          SF_REQUIRE(rc == SF_OK, rc, sf_last_error(c));
          rc = sf_efield(c, nullptr, nullptr);
          SF_REQUIRE(rc == SF_OK, rc, sf_last_error(c));
          solve_ms[i] = ss.ms;
          newton[i] = ss.newton_it;
        } catch (const sf::Error& e) {
          fail(i, e.what());
        } catch (const std::exception& e) {
          fail(i, e.what());
        }
      }
    });
    SF_REQUIRE(errs.empty(), SF_ERR_CUDA, errs);
    for (int i = 0; i < b->n; i++) {
      field_sum += solve_ms[i];
      field_max = std::max(field_max, solve_ms[i]);
    }
    }
    float dev_ms = 0.f;
    SF_CUDA(cudaEventElapsedTime(&dev_ms, b->ev0, b->ev1));
    // autotuner bookkeeping
    if (tuning_shape && b->steps > 0) {  // the first step includes the initial sort's cold caches
      b->shape_ms[shape] += dev_ms;
      b->shape_n[shape]++;
      if (b->steps + 1 >= 4 * TRIAL_STEPS + 1) b->shape = pick_best(b->shape_ms, b->shape_n, 4);
    }
    bool tuning_cycles = false;
    for (int k = 0; k < N_BUCKETS; k++) tuning_cycles |= b->cycles[k] < 0;
    if (tuning_cycles && b->steps > 0) {
      double bms[N_BUCKETS] = {0, 0, 0};
      int bn[N_BUCKETS] = {0, 0, 0};
      for (int i = 0; i < b->n; i++) {
        const int bk = bucket_of(b->ctx[i]);
        bms[bk] += solve_ms[i];
        bn[bk]++;
      }
      for (int k = 0; k < N_BUCKETS; k++)
        if (b->cycles[k] < 0 && bn[k] > 0) {
          b->cyc_ms[k][tuning_step] += bms[k] / bn[k];
          b->cyc_n[k][tuning_step]++;
        }
      if (b->steps + 1 >= 3 * TRIAL_STEPS + 1)
        for (int k = 0; k < N_BUCKETS; k++)
          if (b->cycles[k] < 0) b->cycles[k] = CYCLE_CHOICES[bn[k] > 0 ? pick_best(b->cyc_ms[k], b->cyc_n[k], 3) : 2];
    }
    // particle counts for the caller
    int ovf = 0;
    std::vector<int64_t> nn(b->n), dd(b->n);
    SF_CUDA(cudaMemcpyAsync(nn.data(), b->d.n_dev, 8 * (size_t)b->n, cudaMemcpyDeviceToHost, b->stream));
    SF_CUDA(cudaMemcpyAsync(dd.data(), b->d.dead_dev, 8 * (size_t)b->n, cudaMemcpyDeviceToHost, b->stream));
    SF_CUDA(cudaMemcpyAsync(&ovf, b->d.overflow, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    SF_CUDA(cudaStreamSynchronize(b->stream));
    for (int i = 0; i < b->n; i++) {  // host bookkeeping follows the device counts
      SfSpecies* sp = get_species(b->ctx[i], b->sid[i]);
      sp->n = nn[i];
      sp->cur.n = nn[i];
      sp->n_dead = dd[i];
      sp->sorted = false;
    }
    b->steps++;
    if (st) {
      st->particles = 0;
      st->solve_ms_sum = field_sum;
      st->solve_ms_max = field_max;
      st->newton_it_mean = 0;
      st->newton_it_max = 0;
      for (int i = 0; i < b->n; i++) {
        st->particles += nn[i] - dd[i];
        st->newton_it_mean += newton[i];
        st->newton_it_max = std::max(st->newton_it_max, newton[i]);
      }
      st->newton_it_mean /= b->n;
      st->device_phase_ms = dev_ms;
      st->capacity_overflow = ovf;
    }
    SF_REQUIRE(!ovf, SF_ERR_OOM, "an instance's source exceeded its particle capacity");
    return SF_OK;
  } catch (const sf::Error& e) {
    if (b) b->err = e.what();
    return e.code;
  }
}

int sf_batch_tuning(const sf_batch* b, int32_t* blocks_per_sm, int32_t* slow_blocks, int32_t* cycles_by_bucket) {
  if (!b) return SF_ERR_ARG;
  const int s = b->shape < 0 ? 0 : b->shape;
  if (blocks_per_sm) *blocks_per_sm = b->shape < 0 ? -1 : SHAPES[s][0];
  if (slow_blocks) *slow_blocks = b->shape < 0 ? -1 : SHAPES[s][1];
  if (cycles_by_bucket)
    for (int k = 0; k < N_BUCKETS; k++) cycles_by_bucket[k] = b->cycles[k];
  return SF_OK;
}

}  // extern "C"
