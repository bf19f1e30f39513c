// Range noise: Gaussian, range-relative Gaussian and uniform "dust" returns,
// applied in place to a Ranges buffer.
//
// Replaces rmagine's GaussianNoiseCuda / RelGaussianNoiseCuda /
// UniformDustNoiseCuda (src/rmagine_cuda/src/noise/*.cu; CPU twins in
// src/rmagine_core/src/noise/*.cpp).  Their per-element arithmetic is kept:
//   gaussian:      r <= max_range:  r += z * stddev + mean
//   rel gaussian:  r <= max_range:  r += z * (stddev * r^range_exp) + mean
//   dust:          r' = min(r, max_range); p_hit = 1 - (1 - hit_p)^r';
//                  u0 < p_hit:  d = u1 * r'; u2 < ret_p^d:  r = d
// The random numbers differ by design: the reference keeps one 48-byte
// curandState per element (6.3 GB for a 131 M-ray batch) and advances it;
// here every number is a pure function of (seed, call, element) through the
// counter-based Philox4x32-10 generator (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC 2011), so no state is stored and the
// result does not depend on the launch shape.  A noise object's call counter
// advances per apply, giving fresh numbers each call like the reference's
// advancing states.  Uniforms are odd multiples of 2^-24 in (0, 1); normals
// come from Box-Muller on pairs of uniforms.
//
// Gaussian kinds draw one Philox block (4 numbers -> 4 normals) per group of 4
// consecutive elements (counter = group index); dust draws one block per
// element (counter = element index).  The buffer is streamed once, 8 bytes per
// element.  A 16-byte aligned buffer goes through k_noise_tma: each CTA keeps
// a ring of 16 KiB chunks in shared memory that the bulk-copy (TMA) engine
// fills ahead of the computation and drains with bulk stores, so two chunks
// per CTA are loading while one is computed, whatever the registers allow
// (759 Granges/s = 6.07 TB/s, 90% of the measured HBM copy rate, against 614
// for the register path); the ragged tail and unaligned buffers take k_noise,
// which loads and stores from registers.
#include "internal.h"

namespace rmg {
namespace {

struct U4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

// Philox4x32 with 10 rounds (Salmon et al. 2011, section 3.3 constants).
__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += W0; k1 += W1; }
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(M0, c.x, hi0, lo0);
    mulhilo(M1, c.z, hi1, lo1);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

__device__ __forceinline__ float uniform01(uint32_t x) {
  return __fmul_rn((float)((x >> 8) | 1u), 5.9604644775390625e-08f);  // odd k * 2^-24, exact
}

// Box-Muller: (u1, u2) -> two standard normals, on the special-function unit
// (PTX lg2/sqrt/sin/cos .approx: relative error of lg2 below 2^-22, absolute
// error of sin/cos below 2^-20 on [-pi, pi]), which leaves each normal within
// about 1e-6 of the exact transform of the same uniforms -- far inside the
// noise it models -- at a third of the instructions of the correctly rounded
// functions.  u1 is in (0, 1): log(u1) = lg2(u1) * ln 2 is finite and <= 0.
#ifndef RMG_NOISE_APPROX
#define RMG_NOISE_APPROX 1
#endif
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sin_approx(float x) {
  float y;
  asm("sin.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float cos_approx(float x) {
  float y;
  asm("cos.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void box_muller(float u1, float u2, float& z0, float& z1) {
#if RMG_NOISE_APPROX
  const float r = sqrt_approx(-1.38629436f * lg2_approx(u1));  // -2 ln 2 * log2(u1)
  // angle 2 pi u2 - pi in [-pi, pi): the same circle point up to a half turn, i.e. (-cos, -sin)
  const float a = fmaf(6.28318531f, u2, -3.14159265f);
  z0 = -r * cos_approx(a);
  z1 = -r * sin_approx(a);
#else
  const float r = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  z0 = r * c;
  z1 = r * s;
#endif
}

struct NoiseDev {
  uint32_t kind;
  float mean, stddev, range_exp, hit_p, ret_p, max_range;
  uint32_t key0, key1;      // seed
  uint32_t call0, call1;    // call counter (Philox counter words 2, 3)
};

__device__ __forceinline__ float gauss_one(const NoiseDev& p, float r, float z) {
  if (!(r <= p.max_range)) return r;
  float sd = p.stddev;
  if (p.kind == RMG_NOISE_REL_GAUSSIAN) sd = __fmul_rn(p.stddev, powf(r, p.range_exp));
  return __fadd_rn(r, __fadd_rn(__fmul_rn(z, sd), p.mean));
}

__device__ __forceinline__ float dust_one(const NoiseDev& p, float r, uint64_t i) {
  const U4 b = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), p.call0, p.call1}, p.key0, p.key1);
  const float range = r > p.max_range ? p.max_range : r;
  const float p_hit = (float)(1.0 - (double)powf((float)(1.0 - (double)p.hit_p), range));
  if (uniform01(b.x) < p_hit) {
    const float nr = __fmul_rn(uniform01(b.y), range);
    const float p_ret = powf(p.ret_p, nr);
    if (uniform01(b.z) < p_ret) return nr;
  }
  return r;
}

// Noise of one group of four consecutive ranges (group index g, first element 4 g).
__device__ __forceinline__ void noise_group(const NoiseDev& p, uint64_t g, float v[4]) {
  const uint64_t i0 = 4 * g;
  if (p.kind == RMG_NOISE_UNIFORM_DUST) {
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = dust_one(p, v[k], i0 + k);
  } else {
    const U4 b = philox4x32_10(U4{(uint32_t)g, (uint32_t)(g >> 32), p.call0, p.call1}, p.key0, p.key1);
    float z[4];
    box_muller(uniform01(b.x), uniform01(b.y), z[0], z[1]);
    box_muller(uniform01(b.z), uniform01(b.w), z[2], z[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = gauss_one(p, v[k], z[k]);
  }
}

// Resident CTAs per SM requested from the compiler: 4 (64 registers) measured
// best; 6 (40 registers) and 8 spill and lose (607 / 551 / 388 Granges/s).
#ifndef RMG_NOISE_MIN_BLOCKS
#define RMG_NOISE_MIN_BLOCKS 4
#endif

// Grid-stride over the groups g0, g0 + 1, ... of four ranges: with a 16-byte
// aligned buffer the full groups stream as float4 (a second load kept in flight
// per thread measured slower: 560 against 600 Granges/s); the last partial
// group, and every group of an unaligned buffer, take scalar accesses.
__global__ void __launch_bounds__(256, RMG_NOISE_MIN_BLOCKS) k_noise(float* data, uint64_t n, uint64_t g0,
                                                                    const NoiseDev p) {
  const uint64_t groups = (n + 3) / 4;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool vec = (reinterpret_cast<uintptr_t>(data) & 15u) == 0;
  const uint64_t full_groups = vec ? n / 4 : 0;
  float4* d4 = reinterpret_cast<float4*>(data);
  for (uint64_t g = g0 + tid; g < full_groups; g += stride) {
    const float4 q = __ldcs(d4 + g);
    float v[4] = {q.x, q.y, q.z, q.w};
    noise_group(p, g, v);
    __stcs(d4 + g, make_float4(v[0], v[1], v[2], v[3]));
  }
  for (uint64_t g = (full_groups > g0 ? full_groups : g0) + tid; g < groups; g += stride) {
    const uint64_t i0 = 4 * g;
    float v[4];
    for (int k = 0; k < 4; ++k) v[k] = i0 + k < n ? data[i0 + k] : 0.0f;
    noise_group(p, g, v);
    for (int k = 0; k < 4; ++k)
      if (i0 + k < n) data[i0 + k] = v[k];
  }
}

// ---- bulk-copy (TMA) stream pipeline ----------------------------------------
// Chunk c holds the groups [c * kChunkF4, (c + 1) * kChunkF4): 16 KiB, four
// float4 per thread.  CTA b takes the chunks b, b + grid, b + 2 grid, ...; its ring has
// kStages slots, one mbarrier each.  Thread 0 issues the bulk load of a chunk
// into a free slot (arrive.expect_tx + cp.async.bulk, completing on the slot's
// mbarrier), every thread waits for the slot's phase, noises its float4s in
// shared memory, and after a CTA barrier thread 0 bulk-stores the slot back to
// the same place in global memory.  A slot is loaded again only once the store
// that drains it has finished reading it (cp.async.bulk.wait_group.read), so
// kStages - 1 loads and up to two stores per CTA are in flight.  Measured on
// 131 M ranges (Granges/s, vec / stages / CTAs per SM): 4/3/4 759, 4/4/3 750,
// 2/4/5 709, 2/4/6 717, 8/3/2 672, 1/8/6 580, 4/2/6 596; two stages leave one
// load in flight and lose.
#ifndef RMG_NOISE_TMA_VEC
#define RMG_NOISE_TMA_VEC 4
#endif
#ifndef RMG_NOISE_TMA_STAGES
#define RMG_NOISE_TMA_STAGES 3
#endif
constexpr int kTmaThreads = 256;
constexpr int kTmaVec = RMG_NOISE_TMA_VEC;              // float4 per thread per chunk
constexpr int kChunkF4 = kTmaThreads * kTmaVec;         // 1024 float4 = 4096 ranges
constexpr uint32_t kChunkBytes = kChunkF4 * 16u;        // 16 KiB
constexpr int kStages = RMG_NOISE_TMA_STAGES;
constexpr size_t kRingBytes = (size_t)kStages * kChunkBytes;
// try_wait polls before a slot's load counts as lost (far beyond any real copy:
// a chunk lands within microseconds); the kernel then records RMG_ERR_TIMEOUT
// in the noise status word instead of waiting on.
constexpr unsigned kWaitPolls = 1u << 22;

#ifndef RMG_NOISE_TMA
#define RMG_NOISE_TMA 1
#endif
// Resident CTAs per SM of k_noise_tma (48 KiB ring each).
#ifndef RMG_NOISE_TMA_BLOCKS
#define RMG_NOISE_TMA_BLOCKS 4
#endif

__device__ unsigned int g_noise_status;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "n"(kChunkBytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "n"(kChunkBytes), "r"(bar) : "memory");
}

// Waits for the given phase parity of an mbarrier, at most kWaitPolls polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (unsigned i = 0; i < kWaitPolls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void bulk_store(void* dst, uint32_t src) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "n"(kChunkBytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__global__ void __launch_bounds__(kTmaThreads, RMG_NOISE_TMA_BLOCKS) k_noise_tma(float4* data, uint64_t n_chunks,
                                                                                 const NoiseDev p) {
  extern __shared__ __align__(128) float4 ring_smem[];
  float4 (*ring)[kChunkF4] = reinterpret_cast<float4 (*)[kChunkF4]>(ring_smem);
  __shared__ alignas(8) unsigned long long full[kStages];
  const uint32_t tid = threadIdx.x;
  const uint64_t first = blockIdx.x, step = gridDim.x;
  if (first >= n_chunks) return;  // the whole CTA
  const uint64_t cnt = (n_chunks - first + step - 1) / step;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(smem_u32(&full[s]));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0)
    for (uint64_t j = 0; j < cnt && j < kStages - 1; ++j)
      bulk_load(smem_u32(ring[j]), data + (first + j * step) * kChunkF4, smem_u32(&full[j]));
  uint64_t i = 0;
  bool failed = false;
  for (; i < cnt; ++i) {
    const int s = (int)(i % kStages);
    const bool ok = mbar_wait(smem_u32(&full[s]), (uint32_t)(i / kStages) & 1u);
    const uint64_t c = first + i * step;
#pragma unroll
    for (int u = 0; u < kTmaVec; ++u) {
      float4* q = &ring[s][u * kTmaThreads + tid];
      const float4 x = *q;
      float v[4] = {x.x, x.y, x.z, x.w};
      noise_group(p, c * kChunkF4 + (uint64_t)(u * kTmaThreads + tid), v);
      *q = make_float4(v[0], v[1], v[2], v[3]);
    }
    // The bulk store reads the slot through the async proxy.
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (__syncthreads_or(!ok)) {  // uniform: a lost load ends the CTA's work, unstored
      failed = true;
      break;
    }
    if (tid == 0) {
      bulk_store(data + c * kChunkF4, smem_u32(ring[s]));
      const uint64_t j = i + kStages - 1;
      if (j < cnt) {
        // Slot j % kStages was drained by the store issued one iteration ago.
        asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        const int sj = (int)(j % kStages);
        bulk_load(smem_u32(ring[sj]), data + (first + j * step) * kChunkF4, smem_u32(&full[sj]));
      }
    }
  }
  if (tid == 0) {
    if (failed) {
      atomicExch(&g_noise_status, (unsigned)RMG_ERR_TIMEOUT);
      // Loads of the chunks i .. i + kStages - 2 may still be landing in the ring.
      for (uint64_t j = i; j < cnt && j < i + kStages - 1; ++j)
        mbar_wait(smem_u32(&full[j % kStages]), (uint32_t)(j / kStages) & 1u);
    }
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
}

// The raw generator for tests: out[4*i .. 4*i+3] = philox(counter i, call, seed).
__global__ void k_philox_raw(uint32_t* out, uint64_t n_blocks, const NoiseDev p) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_blocks) return;
  const U4 b = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), p.call0, p.call1}, p.key0, p.key1);
  out[4 * i] = b.x; out[4 * i + 1] = b.y; out[4 * i + 2] = b.z; out[4 * i + 3] = b.w;
}

int to_dev(const rmg_noise* noise, NoiseDev& p) {
  if (!noise) return fail(RMG_ERR_INVALID_ARG, "noise: NULL parameters");
  if (noise->kind > RMG_NOISE_UNIFORM_DUST) return fail(RMG_ERR_INVALID_ARG, "noise: unknown kind");
  p.kind = noise->kind;
  p.mean = noise->mean;
  p.stddev = noise->stddev;
  p.range_exp = noise->range_exp;
  p.hit_p = noise->hit_probability;
  p.ret_p = noise->return_probability;
  p.max_range = noise->max_range;
  p.key0 = (uint32_t)noise->seed;
  p.key1 = (uint32_t)(noise->seed >> 32);
  p.call0 = (uint32_t)noise->call;
  p.call1 = (uint32_t)(noise->call >> 32);
  return RMG_OK;
}

}  // namespace
}  // namespace rmg

using namespace rmg;

extern "C" int rmg_noise_apply(const rmg_noise* noise, float* ranges, uint64_t n, void* stream) {
  return guarded("rmg_noise_apply", [&]() -> int {
    NoiseDev p;
    int s = to_dev(noise, p);
    if (s != RMG_OK) return s;
    if (n == 0) return RMG_OK;
    if (!ranges) return fail(RMG_ERR_INVALID_ARG, "rmg_noise_apply: ranges is NULL");
    const uint64_t groups = (n + 3) / 4;
    uint64_t g0 = 0;
    cudaStream_t st = as_stream(stream);
    if (RMG_NOISE_TMA && (reinterpret_cast<uintptr_t>(ranges) & 15u) == 0) {
      const uint64_t n_chunks = (n / 4) / kChunkF4;
      if (n_chunks > 0) {
        static thread_local int attr_device = -1;  // the ring may exceed the 48 KB default
        int dev = 0;
        RMG_CUDA_TRY(cudaGetDevice(&dev));
        if (attr_device != dev) {
          RMG_CUDA_TRY(cudaFuncSetAttribute(k_noise_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes));
          attr_device = dev;
        }
        const uint64_t cap = (uint64_t)RMG_NOISE_TMA_BLOCKS * (uint64_t)device_sm_count();  // resident CTAs
        k_noise_tma<<<(unsigned)(n_chunks < cap ? n_chunks : cap), kTmaThreads, kRingBytes, st>>>(
            reinterpret_cast<float4*>(ranges), n_chunks, p);
        s = cuda_status(cudaGetLastError(), "k_noise_tma");
        if (s != RMG_OK) return s;
        g0 = n_chunks * kChunkF4;
      }
    }
    if (g0 == groups) return RMG_OK;
    const uint64_t want = (groups - g0 + 255) / 256;
    const uint64_t cap = 8ull * (uint64_t)device_sm_count();  // grid-stride beyond this
    const unsigned grid = (unsigned)(want < cap ? want : cap);
    k_noise<<<grid, 256, 0, st>>>(ranges, n, g0, p);
    return cuda_status(cudaGetLastError(), "k_noise");
  });
}

extern "C" int rmg_noise_status(uint32_t* status, int clear) {
  return guarded("rmg_noise_status", [&]() -> int {
    if (!status) return fail(RMG_ERR_INVALID_ARG, "rmg_noise_status: status is NULL");
    unsigned v = 0;
    RMG_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_noise_status, sizeof v));
    *status = v;
    if (clear) {
      const unsigned zero = 0;
      RMG_CUDA_TRY(cudaMemcpyToSymbol(g_noise_status, &zero, sizeof zero));
    }
    return RMG_OK;
  });
}

extern "C" int rmg_noise_philox(const rmg_noise* noise, uint32_t* out, uint64_t n_blocks, void* stream) {
  return guarded("rmg_noise_philox", [&]() -> int {
    NoiseDev p;
    int s = to_dev(noise, p);
    if (s != RMG_OK) return s;
    if (n_blocks == 0) return RMG_OK;
    if (!out) return fail(RMG_ERR_INVALID_ARG, "rmg_noise_philox: out is NULL");
    k_philox_raw<<<(unsigned)((n_blocks + 255) / 256), 256, 0, as_stream(stream)>>>(out, n_blocks, p);
    return cuda_status(cudaGetLastError(), "k_philox_raw");
  });
}
