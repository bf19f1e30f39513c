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
// element (counter = element index).  The kernel streams the buffer once with
// 16-byte accesses, 8 bytes per element; the generator's integer multiplies
// and the stream's latency bound it, at about 70% of the HBM roof.
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
#pragma unroll
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

// Grid-stride over groups of four ranges: with a 16-byte aligned buffer the full
// groups stream as float4 (a second load kept in flight per thread measured
// slower: 560 against 600 Granges/s); the last partial group, and every group
// of an unaligned buffer, take scalar accesses.
__global__ void __launch_bounds__(256, RMG_NOISE_MIN_BLOCKS) k_noise(float* data, uint64_t n, const NoiseDev p) {
  const uint64_t groups = (n + 3) / 4;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool vec = (reinterpret_cast<uintptr_t>(data) & 15u) == 0;
  const uint64_t full_groups = vec ? n / 4 : 0;
  float4* d4 = reinterpret_cast<float4*>(data);
  for (uint64_t g = tid; g < full_groups; g += stride) {
    const float4 q = __ldcs(d4 + g);
    float v[4] = {q.x, q.y, q.z, q.w};
    noise_group(p, g, v);
    __stcs(d4 + g, make_float4(v[0], v[1], v[2], v[3]));
  }
  for (uint64_t g = full_groups + tid; g < groups; g += stride) {
    const uint64_t i0 = 4 * g;
    float v[4];
    for (int k = 0; k < 4; ++k) v[k] = i0 + k < n ? data[i0 + k] : 0.0f;
    noise_group(p, g, v);
    for (int k = 0; k < 4; ++k)
      if (i0 + k < n) data[i0 + k] = v[k];
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
  NoiseDev p;
  int s = to_dev(noise, p);
  if (s != RMG_OK) return s;
  if (n == 0) return RMG_OK;
  if (!ranges) return fail(RMG_ERR_INVALID_ARG, "rmg_noise_apply: ranges is NULL");
  const uint64_t groups = (n + 3) / 4;
  const uint64_t want = (groups + 255) / 256;
  const uint64_t cap = 8ull * (uint64_t)device_sm_count();  // grid-stride beyond this
  const unsigned grid = (unsigned)(want < cap ? want : cap);
  k_noise<<<grid, 256, 0, as_stream(stream)>>>(ranges, n, p);
  return cuda_status(cudaGetLastError(), "k_noise");
}

extern "C" int rmg_noise_philox(const rmg_noise* noise, uint32_t* out, uint64_t n_blocks, void* stream) {
  NoiseDev p;
  int s = to_dev(noise, p);
  if (s != RMG_OK) return s;
  if (n_blocks == 0) return RMG_OK;
  if (!out) return fail(RMG_ERR_INVALID_ARG, "rmg_noise_philox: out is NULL");
  k_philox_raw<<<(unsigned)((n_blocks + 255) / 256), 256, 0, as_stream(stream)>>>(out, n_blocks, p);
  return cuda_status(cudaGetLastError(), "k_philox_raw");
}
