// sf_conv_tc.cu -- 3x3 convolutions of the learned Poisson start on the fifth-generation
// tensor cores (tcgen05): TMA tile loads into swizzled shared memory, tcgen05.mma with the
// accumulator in tensor memory, tcgen05.ld for the epilogue.  (No reference counterpart:
// the network exists only in this build.)
//
// Implicit GEMM: D[pixel][co] = sum over taps (ky, kx) and input channels ci of
// in[y + ky - 1][x + kx - 1][ci] * w[co][ky][kx][ci].  One CTA computes M = 128 pixels (a
// box of BW x BH pixels, BW * BH = 128) by N output channels.  The K loop runs over the 9
// taps and the input channels in chunks of CK (16, 32 or 64 channels, one swizzle atom
// row of 32, 64 or 128 bytes): per step the TMA loads the A box (CK x BW x BH, shifted by
// the tap; coordinates outside the image read as zero, which is the convolution's zero
// padding) and the B box (CK x N of the weights, K-major), and CK / 16 MMAs of
// M128 x N x K16 accumulate into tensor memory.
//
// Roles in the CTA (128 threads): thread 0 issues the TMA loads into a ring of stages,
// thread 32 issues the MMAs, and all four warps read the accumulator back (warp w holds
// tensor-memory lanes 32w..32w+31, i.e. pixels 32w..32w+31) and write bias + ReLU as
// BF16.  Every wait on an mbarrier is bounded (2 s): on timeout the CTA records an error,
// stops issuing, waits (bounded again) for the copies and MMAs it has in flight, and still
// frees its tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "sf_internal.h"

using namespace sf;
typedef __nv_bfloat16 bf16;

namespace {

constexpr int TC_THREADS = 128;
constexpr int TC_M = 128;
constexpr unsigned long long WAIT_NS = 2000000000ull;  // a wait longer than 2 s counts as failed
constexpr int TC_SMEM_LIMIT = 210 * 1024;  // dynamic shared memory of every launch: <= 200 KB of stages + 1 KB

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// bounded wait for the phase with the given parity; false after limit_ns
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned long long limit_ns) {
  const uint32_t a = smem_u32(bar);
  const unsigned long long t0 = global_ns();
  for (unsigned k = 0;; k++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((k & 63) == 63 && global_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile whose rows are one swizzle
// atom wide (S = 32, 64 or 128 bytes, rows contiguous): start address, stride between
// 8-row groups (8 S), descriptor version 1, swizzle mode (6: 32 B, 4: 64 B, 2: 128 B).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int swz_bytes) {
  const uint64_t mode = swz_bytes == 128 ? 2 : (swz_bytes == 64 ? 4 : 6);
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                                  // leading-dimension offset (unused here)
  d |= (uint64_t)(((8 * swz_bytes) >> 4) & 0x3FFF) << 32;  // stride between 8-row groups
  d |= (uint64_t)1 << 46;                                  // descriptor version
  d |= mode << 61;
  return d;
}

// Instruction descriptor of tcgen05.mma.kind::f16: D FP32, A and B BF16, both K-major,
// M = 128, N as given.
__host__ __device__ constexpr uint32_t instr_desc(int n) {
  return (1u << 4)                     // D: F32
         | (1u << 7)                   // A: BF16
         | (1u << 10)                  // B: BF16
         | ((uint32_t)(n >> 3) << 17)  // N / 8
         | ((uint32_t)(TC_M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_bf16_tmem(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

struct TcArgs {
  const float* bias;
  bf16* out;
  int H, W, Cin, Cout, out_C, out_c0, relu;
  int BW, BH;     // pixel box: BW x BH = 128
  int CK;         // input channels per K step
  int N;          // output channels per CTA
  int tmem_cols;  // power of two >= max(32, N)
  int stages;
  int* err;
  unsigned long long wait_ns;  // limit of each mbarrier wait (WAIT_NS)
  int stall;                   // wait test: no copy is issued, so the first wait runs out
};

// One CTA: output pixels of box (blockIdx.x, blockIdx.y), channels [blockIdx.z N, +N).
__global__ void __launch_bounds__(TC_THREADS, 1) k_conv3x3_tc(const __grid_constant__ CUtensorMap map_a,
                                                               const __grid_constant__ CUtensorMap map_b, TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[8];
  __shared__ __align__(8) uint64_t empty_bar[8];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // stage buffers start on a 1024-byte boundary (the 128-byte swizzle repeats every 8 rows)
  unsigned char* base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  const int a_bytes = TC_M * a.CK * 2, b_bytes = a.N * a.CK * 2;
  const int stage_bytes = ((a_bytes + b_bytes + 1023) / 1024) * 1024;
  const int swz = a.CK * 2;
  const int x0 = blockIdx.x * a.BW, y0 = blockIdx.y * a.BH, co0 = blockIdx.z * a.N;
  const int kchunks = a.Cin / a.CK, ksteps = 9 * kchunks;

  if (tid == 0) {
    for (int s = 0; s < a.stages; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(a.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  int last_load = -1, last_mma = -1;  // the last step whose copies / MMAs this thread issued

  if (tid == 0 && !a.stall) {
    // producer: the A box of the step's tap and channel chunk, and the B box of weights
    for (int k = 0; k < ksteps; k++) {
      const int s = k % a.stages, use = k / a.stages;
      if (use > 0 && !mbar_wait(&empty_bar[s], (use - 1) & 1, a.wait_ns)) {
        atomicExch(&failed, 1);
        break;
      }
      if (*(volatile int*)&failed) break;
      const int tap = k / kchunks, ci0 = (k % kchunks) * a.CK;
      const int ky = tap / 3, kx = tap % 3;
      unsigned char* st = base + s * stage_bytes;
      mbar_expect_tx(&full_bar[s], (unsigned)(a_bytes + b_bytes));
      tma_load_3d(st, &map_a, ci0, x0 + kx - 1, y0 + ky - 1, &full_bar[s]);
      tma_load_2d(st + a_bytes, &map_b, tap * a.Cin + ci0, co0, &full_bar[s]);
      last_load = k;
    }
  } else if (tid == 32) {
    // MMA issuer
    const uint32_t idesc = instr_desc(a.N);
    bool ok = true;
    for (int k = 0; k < ksteps; k++) {
      const int s = k % a.stages, use = k / a.stages;
      if (!mbar_wait(&full_bar[s], use & 1, a.wait_ns)) {
        atomicExch(&failed, 1);
        ok = false;
        break;
      }
      if (*(volatile int*)&failed) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = smem_u32(base + s * stage_bytes);
      const uint32_t sb = sa + a_bytes;
      for (int kk = 0; kk < a.CK / 16; kk++) {
        // K = 16 BF16 = 32 bytes further along the swizzled rows
        const uint64_t da = smem_desc(sa + 32 * kk, swz), db = smem_desc(sb + 32 * kk, swz);
        mma_bf16_tmem(tmem, da, db, idesc, (k > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
      last_mma = k;
    }
    if (ok) mma_commit(&done_bar);
    else mbar_expect_tx(&done_bar, 0);  // release the epilogue without a result
  }
  __syncwarp();

  // epilogue: every warp waits for the accumulator, then reads its 32 lanes (pixels)
  // (longer than the MMA issuer's own waits, which end by releasing this barrier)
  const bool done = mbar_wait(&done_bar, 0, 4 * a.wait_ns);
  if (!done) atomicExch(&failed, 1);  // a wait that ran out here is an error too
  const bool have = done && !*(volatile int*)&failed;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (have) {
    const int p = 32 * warp + lane;
    const int x = x0 + p % a.BW, y = y0 + p / a.BW;
    const bool in_img = x < a.W && y < a.H;
    bf16* op = a.out + ((size_t)y * a.W + x) * a.out_C + a.out_c0 + co0;
    for (int c = 0; c < a.N; c += 16) {
      uint32_t r[16];
      const uint32_t addr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (!in_img) continue;
      __align__(16) __nv_bfloat162 v[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float f0 = __uint_as_float(r[2 * q]), f1 = __uint_as_float(r[2 * q + 1]);
        if (a.bias) {
          f0 += a.bias[co0 + c + 2 * q];
          f1 += a.bias[co0 + c + 2 * q + 1];
        }
        if (a.relu) {
          f0 = fmaxf(f0, 0.f);
          f1 = fmaxf(f1, 0.f);
        }
        v[q] = __floats2bfloat162_rn(f0, f1);
      }
      uint4* dst = reinterpret_cast<uint4*>(op + c);
      dst[0] = reinterpret_cast<const uint4*>(v)[0];
      dst[1] = reinterpret_cast<const uint4*>(v)[1];
    }
  }
  // after a timeout, nothing this CTA started may still be running when it frees its tensor
  // memory and exits: the producer waits (bounded) for the copies of its last stages, the
  // MMA issuer for its last commit (which covers every MMA it issued before)
  if (*(volatile int*)&failed) {
    if (tid == 0)
      for (int k = max(0, last_load - a.stages + 1); k <= last_load; k++)
        mbar_wait(&full_bar[k % a.stages], (unsigned)(k / a.stages) & 1u, a.wait_ns);
    if (tid == 32 && last_mma >= 0)
      mbar_wait(&empty_bar[last_mma % a.stages], (unsigned)(last_mma / a.stages) & 1u, a.wait_ns);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid == 0 && failed) atomicExch(a.err, 1);
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_encode_mutex;

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  std::lock_guard<std::mutex> lock(g_encode_mutex);
  if (!g_encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    SF_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    SF_REQUIRE(q == cudaDriverEntryPointSuccess && fn, SF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  return g_encode;
}

CUtensorMapSwizzle swizzle_of(int bytes) {
  return bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : (bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

int pick_ck(int cin) { return cin % 64 == 0 ? 64 : (cin % 32 == 0 ? 32 : 16); }

}  // namespace

namespace sf {

// The shapes the tensor-core path takes: channels in multiples of 16, rows of 16, 32, 64 or
// a multiple of 128 pixels (a 128-pixel box then covers whole rows or part of one row),
// and an output channel slice on a 16-byte boundary.
bool conv3x3_tc_supported(int H, int W, int Cin, int Cout, int out_C, int out_c0) {
  if (Cin < 16 || Cin % 16 != 0 || Cout < 16 || Cout % 16 != 0) return false;
  if (!(W == 16 || W == 32 || W == 64 || W % 128 == 0)) return false;
  if (out_c0 % 8 != 0 || out_C % 8 != 0) return false;
  return H >= 1;
}

// out[y][x][out_c0 + co] = act(bias[co] + sum w[co][ky][kx][ci] in[y+ky-1][x+kx-1][ci]) on
// the tensor cores.  in: H x W x Cin BF16 (NHWC), w: Cout x 9 x Cin BF16.  err: device int
// set to 1 if a CTA's pipeline timed out (the output is then incomplete).
static void conv3x3_tc_launch(cudaStream_t s, const bf16* in, int H, int W, int Cin, const bf16* w,
                              const float* bias, int Cout, bf16* out, int out_C, int out_c0, bool relu, int* err,
                              unsigned long long wait_ns, bool stall) {
  SF_REQUIRE(conv3x3_tc_supported(H, W, Cin, Cout, out_C, out_c0), SF_ERR_ARG, "shape not on the tensor-core path");
  TcArgs a{};
  a.wait_ns = wait_ns;
  a.stall = stall ? 1 : 0;
  a.bias = bias;
  a.out = out;
  a.H = H;
  a.W = W;
  a.Cin = Cin;
  a.Cout = Cout;
  a.out_C = out_C;
  a.out_c0 = out_c0;
  a.relu = relu ? 1 : 0;
  a.BW = W >= 128 ? 128 : W;
  a.BH = TC_M / a.BW;
  a.CK = pick_ck(Cin);
  // output channels per CTA: all of them up to 256, else the largest multiple of 16 that
  // divides Cout and is at most 128
  int n = Cout;
  if (n > 256) {
    n = 128;
    while (Cout % n != 0) n -= 16;
  }
  a.N = n;
  a.tmem_cols = 32;
  while (a.tmem_cols < a.N) a.tmem_cols <<= 1;
  a.err = err;
  const int a_bytes = TC_M * a.CK * 2, b_bytes = a.N * a.CK * 2;
  const int stage_bytes = ((a_bytes + b_bytes + 1023) / 1024) * 1024;
  a.stages = std::max(2, std::min(6, (200 * 1024) / stage_bytes));
  const size_t smem = (size_t)a.stages * stage_bytes + 1024;

  auto enc = encoder();
  CUtensorMap ma, mb;
  {
    // A: (C, W, H) with C contiguous; box (CK, BW, BH)
    const cuuint64_t dims[3] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H};
    const cuuint64_t strides[2] = {(cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2};
    const cuuint32_t box[3] = {(cuuint32_t)a.CK, (cuuint32_t)a.BW, (cuuint32_t)a.BH};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = enc(&ma, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(in), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(a.CK * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SF_REQUIRE(r == CUDA_SUCCESS, SF_ERR_CUDA, "cuTensorMapEncodeTiled (activations) failed");
  }
  {
    // B: weights as (9 Cin, Cout) with the 9 Cin taps-and-channels contiguous; box (CK, N)
    const cuuint64_t dims[2] = {(cuuint64_t)9 * Cin, (cuuint64_t)Cout};
    const cuuint64_t strides[1] = {(cuuint64_t)9 * Cin * 2};
    const cuuint32_t box[2] = {(cuuint32_t)a.CK, (cuuint32_t)a.N};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(w), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(a.CK * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SF_REQUIRE(r == CUDA_SUCCESS, SF_ERR_CUDA, "cuTensorMapEncodeTiled (weights) failed");
  }
  // the shared-memory limit is set once per device, to a bound above every launch's need,
  // so that launches captured into CUDA graphs make no attribute call
  {
    static std::mutex m;
    static bool set[64] = {};
    int dev = 0;
    SF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(m);
    if (dev < 0 || dev >= 64 || !set[dev]) {
      SF_CUDA(cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_LIMIT));
      if (dev >= 0 && dev < 64) set[dev] = true;
    }
  }
  SF_REQUIRE(smem <= (size_t)TC_SMEM_LIMIT, SF_ERR_ARG, "tensor-core convolution stages exceed the shared memory");
  const dim3 grid((W + a.BW - 1) / a.BW, (H + a.BH - 1) / a.BH, Cout / a.N);
  k_conv3x3_tc<<<grid, TC_THREADS, smem, s>>>(ma, mb, a);
  SF_CUDA(cudaGetLastError());
}

void conv3x3_tc(cudaStream_t s, const bf16* in, int H, int W, int Cin, const bf16* w, const float* bias, int Cout,
                bf16* out, int out_C, int out_c0, bool relu, int* err) {
  conv3x3_tc_launch(s, in, H, W, Cin, w, bias, Cout, out, out_C, out_c0, relu, err, WAIT_NS, false);
}

// One 16x16x16 -> 16 convolution in which no copy is issued, so that the MMA issuer's first
// wait runs out (after 20 ms): the CTA has to record the failure, release its epilogue, free
// its tensor memory and return.  Returns the kernel's error flag (1 when the wait ran out).
int conv3x3_tc_wait_test(cudaStream_t s) {
  const int H = 16, W = 16, C = 16;
  bf16 *in = nullptr, *w = nullptr, *out = nullptr;
  int* err = nullptr;
  int herr = -1;
  SF_CUDA(cudaMalloc(&in, sizeof(bf16) * H * W * C));
  SF_CUDA(cudaMalloc(&w, sizeof(bf16) * C * 9 * C));
  SF_CUDA(cudaMalloc(&out, sizeof(bf16) * H * W * C));
  SF_CUDA(cudaMalloc(&err, sizeof(int)));
  try {
    SF_CUDA(cudaMemsetAsync(in, 0, sizeof(bf16) * H * W * C, s));
    SF_CUDA(cudaMemsetAsync(w, 0, sizeof(bf16) * C * 9 * C, s));
    SF_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    conv3x3_tc_launch(s, in, H, W, C, w, nullptr, C, out, C, 0, false, err, 20000000ull, true);
    SF_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SF_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    cudaStreamSynchronize(s);
    cudaFree(in); cudaFree(w); cudaFree(out); cudaFree(err);
    throw;
  }
  SF_CUDA(cudaFree(in));
  SF_CUDA(cudaFree(w));
  SF_CUDA(cudaFree(out));
  SF_CUDA(cudaFree(err));
  return herr;
}

}  // namespace sf
