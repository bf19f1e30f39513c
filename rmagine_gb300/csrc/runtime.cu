// Library runtime: status strings, per-thread error messages, device queries,
// bounded stream waits, and sensor models (device ray-direction tables).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>

#include "internal.h"

namespace rmg {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RMG_OK;
  cudaGetLastError();
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return RMG_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return RMG_ERR_NO_DEVICE;
  return RMG_ERR_CUDA;
}

int device_sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return sms > 0 ? sms : 1;
}

namespace {

// SphericalModel::getDirection (types/sensor_models.h:169-174):
//   phi = phi.min + vid*phi.inc, theta = theta.min + hid*theta.inc  (binary32,
//   multiply then add, no contraction), d = (cosf(phi) cosf(theta),
//   cosf(phi) sinf(theta), sinf(phi)).
// The reference evaluates these with the C library's cosf/sinf, which are not
// correctly rounded (about 2% of arguments differ by one ulp from the
// correctly rounded value), so the table is evaluated once per model with the
// host C library, exactly as the reference's own ray generator does, and
// uploaded.  The H + W trigonometric values are computed once; every ray of
// every pose then reads its direction from device memory.
void dirs_spherical_host(const rmg_discrete_interval& phi, const rmg_discrete_interval& theta,
                         std::vector<float>& out) {
  const uint32_t W = theta.size, H = phi.size;
  out.resize(3ull * W * H);
  std::vector<float> ct(W), st(W);
  for (uint32_t h = 0; h < W; ++h) {
    const volatile float prod = (float)h * theta.inc;  // no contraction into fmaf
    const float t = theta.min + prod;
    ct[h] = cosf(t);
    st[h] = sinf(t);
  }
  for (uint32_t v = 0; v < H; ++v) {
    const volatile float prod = (float)v * phi.inc;
    const float p = phi.min + prod;
    const float cp = cosf(p), sp = sinf(p);
    float* row = out.data() + 3ull * v * W;
    for (uint32_t h = 0; h < W; ++h) {
      row[3 * h + 0] = cp * ct[h];
      row[3 * h + 1] = cp * st[h];
      row[3 * h + 2] = sp;
    }
  }
}

// PinholeModel::getDirectionOptical / getDirection (sensor_models.h:256-276):
//   pX = (hid - cx)/fx, pY = (vid - cy)/fy, v = normalize(pX, pY, 1) with
//   normalize = divide by sqrt(x*x + y*y + z*z); mapped to (z, -x, -y).
__global__ void k_dirs_pinhole(uint32_t W, uint32_t H, float fx, float fy, float cx, float cy,
                               float* dirs) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * H) return;
  const uint32_t vid = i / W, hid = i - vid * W;
  const float px = __fdiv_rn(__fsub_rn(__uint2float_rn(hid), cx), fx);
  const float py = __fdiv_rn(__fsub_rn(__uint2float_rn(vid), cy), fy);
  const float pz = 1.0f;
  const float n2 = __fadd_rn(__fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py)), __fmul_rn(pz, pz));
  const float n = __fsqrt_rn(n2);
  const float x = __fdiv_rn(px, n), y = __fdiv_rn(py, n), z = __fdiv_rn(pz, n);
  dirs[3 * i + 0] = z;
  dirs[3 * i + 1] = -x;
  dirs[3 * i + 2] = -y;
}

void free_sensor(rmg_sensor* s) {
  if (!s) return;
  cudaFree(s->d_dirs);
  cudaFree(s->d_origs);
  cudaFree(s->d_order);
  delete s;
}

// Visiting order of a direction table (O1Dn / OnDn).  A table of directions
// scattered over the sphere (random directions, as in a test pattern) gives
// every warp 32 rays that part at the root, while the same rays sorted by
// elevation band and then azimuth share their paths through the tree: 1.8x
// faster on a 1M-triangle terrain for 10,000 uniform directions.  Bands are
// a quarter of the side of a square holding 32 rays, alternately swept in
// opposite azimuth directions; non-finite or zero directions go last.  The
// sorted order is kept only when it halves the mean 1 - cos of the angle
// between neighbours within groups of 32 rays (a sensor's own beam order is
// usually coherent already); the result is empty otherwise.
std::vector<uint32_t> visiting_order(const float* dirs, size_t n) {
  std::vector<uint32_t> order;
  if (n < 64 || n > (1ull << 26)) return order;
  auto unit = [&](size_t i, double u[3]) -> bool {
    const double x = dirs[3 * i], y = dirs[3 * i + 1], z = dirs[3 * i + 2];
    const double l = std::sqrt(x * x + y * y + z * z);
    if (!(l > 0.0) || !std::isfinite(l)) return false;
    u[0] = x / l; u[1] = y / l; u[2] = z / l;
    return true;
  };
  auto spread = [&](const uint32_t* idx) {
    double sum = 0.0;
    size_t cnt = 0;
    for (size_t i = 0; i + 1 < n; ++i) {
      if ((i & 31) == 31) continue;
      double a[3], b[3];
      if (!unit(idx ? idx[i] : i, a) || !unit(idx ? idx[i + 1] : i + 1, b)) continue;
      sum += 1.0 - (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
      ++cnt;
    }
    return cnt ? sum / (double)cnt : 0.0;
  };
  const double pi = 3.14159265358979323846;
  const double band = std::sqrt(128.0 * pi / (double)n) / 4.0;
  std::vector<std::pair<uint64_t, uint32_t>> key(n);
  for (size_t i = 0; i < n; ++i) {
    double u[3];
    uint64_t k = ~0ull;
    if (unit(i, u)) {
      const double e = std::asin(std::min(1.0, std::max(-1.0, u[2])));
      const uint64_t b = (uint64_t)std::floor((e + pi / 2) / band);
      const double az = std::atan2(u[1], u[0]);
      uint64_t q = (uint64_t)std::min(16777215.0, std::max(0.0, (az + pi) / (2 * pi) * 16777216.0));
      if (b & 1) q = 16777215 - q;
      k = b << 32 | q;
    }
    key[i] = {k, (uint32_t)i};
  }
  std::stable_sort(key.begin(), key.end(),
                   [](const std::pair<uint64_t, uint32_t>& a, const std::pair<uint64_t, uint32_t>& b) {
                     return a.first < b.first;
                   });
  order.resize(n);
  for (size_t i = 0; i < n; ++i) order[i] = key[i].second;
  if (!(spread(order.data()) < 0.5 * spread(nullptr))) order.clear();
  return order;
}

}  // namespace

SensorDev device_view(const rmg_sensor* s) {
  SensorDev d;
  d.kind = s->model.kind;
  d.width = s->width;
  d.height = s->height;
  d.range_min = s->model.range.min;
  d.range_max = s->model.range.max;
  d.dirs = s->d_dirs;
  d.origs = s->d_origs;
  d.orig = make_float3(s->model.orig.x, s->model.orig.y, s->model.orig.z);
  d.order = s->d_order;
  return d;
}

}  // namespace rmg

using namespace rmg;

extern "C" const char* rmg_status_string(int status) {
  switch (status) {
    case RMG_OK: return "ok";
    case RMG_ERR_INVALID_ARG: return "invalid argument";
    case RMG_ERR_CUDA: return "CUDA error";
    case RMG_ERR_OOM: return "out of device memory";
    case RMG_ERR_TIMEOUT: return "timeout";
    case RMG_ERR_TRAVERSAL_BUDGET: return "traversal budget exceeded (corrupt BVH?)";
    case RMG_ERR_NO_DEVICE: return "no usable CUDA device";
    case RMG_ERR_UNSUPPORTED: return "unsupported option";
    default: return "unknown status";
  }
}

extern "C" const char* rmg_last_error(void) { return g_last_error.c_str(); }

extern "C" int rmg_abi_version(void) { return RMG_ABI_VERSION; }

extern "C" int rmg_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  return guarded("rmg_device_info", [&]() -> int {
    int dev = 0;
    RMG_CUDA_TRY(cudaGetDevice(&dev));
    int sms = 0, ma = 0, mi = 0;
    RMG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RMG_CUDA_TRY(cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, dev));
    RMG_CUDA_TRY(cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, dev));
    if (sm_count) *sm_count = sms;
    if (cc_major) *cc_major = ma;
    if (cc_minor) *cc_minor = mi;
    return RMG_OK;
  });
}

extern "C" int rmg_stream_wait(void* stream, uint32_t timeout_ms) {
  return guarded("rmg_stream_wait", [&]() -> int {
    cudaStream_t st = as_stream(stream);
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
      const cudaError_t e = cudaStreamQuery(st);
      if (e == cudaSuccess) return RMG_OK;
      if (e != cudaErrorNotReady) return cuda_status(e, "cudaStreamQuery");
      const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
                          std::chrono::steady_clock::now() - t0).count();
      if ((uint64_t)ms >= timeout_ms) return fail(RMG_ERR_TIMEOUT, "rmg_stream_wait: timed out");
      std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
  });
}

extern "C" int rmg_sensor_create(const rmg_model* model, void* stream, rmg_sensor** out) {
  return guarded("rmg_sensor_create", [&]() -> int {
    if (!out || !model) return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: NULL argument");
    *out = nullptr;
    uint32_t W = 0, H = 0;
    switch (model->kind) {
      case RMG_MODEL_SPHERICAL: W = model->theta.size; H = model->phi.size; break;
      case RMG_MODEL_PINHOLE:
        W = model->width; H = model->height;
        if (!(model->f[0] != 0.0f) || !(model->f[1] != 0.0f))
          return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: pinhole focal length is zero");
        break;
      case RMG_MODEL_O1DN:
      case RMG_MODEL_ONDN:
        W = model->width; H = model->height;
        if (!model->dirs) return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: dirs is NULL");
        if (model->kind == RMG_MODEL_ONDN && !model->origs)
          return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: origs is NULL");
        break;
      default: return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: unknown model kind");
    }
    if (W == 0 || H == 0) return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: empty model");
    if ((uint64_t)W * H > (1ull << 31)) return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: model too large");
    if (!(model->range.max >= model->range.min))
      return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_create: range.max < range.min");
  
    cudaStream_t st = as_stream(stream);
    rmg_sensor* s = new (std::nothrow) rmg_sensor;
    if (!s) return fail(RMG_ERR_OOM, "rmg_sensor_create: host allocation");
    std::memset(s, 0, sizeof(*s));
    cudaGetDevice(&s->device);
    s->model = *model;
    s->model.dirs = nullptr;
    s->model.origs = nullptr;
    s->width = W;
    s->height = H;
    const size_t n = (size_t)W * H;
    int r = dev_alloc(&s->d_dirs, 3 * n, "sensor dirs");
    if (r == RMG_OK && model->kind == RMG_MODEL_ONDN) r = dev_alloc(&s->d_origs, 3 * n, "sensor origs");
    if (r != RMG_OK) { free_sensor(s); return r; }
    const unsigned grid = (unsigned)((n + 255) / 256);
    switch (model->kind) {
      case RMG_MODEL_SPHERICAL: {
        std::vector<float> table;
        dirs_spherical_host(model->phi, model->theta, table);
        r = cuda_status(cudaMemcpyAsync(s->d_dirs, table.data(), 4 * table.size(), cudaMemcpyHostToDevice, st),
                        "copy spherical dirs");
        if (r == RMG_OK) r = cuda_status(cudaStreamSynchronize(st), "sensor sync");
        break;
      }
      case RMG_MODEL_PINHOLE:
        k_dirs_pinhole<<<grid, 256, 0, st>>>(W, H, model->f[0], model->f[1], model->c[0], model->c[1],
                                             s->d_dirs);
        r = cuda_status(cudaGetLastError(), "k_dirs_pinhole");
        break;
      default: {
        r = cuda_status(cudaMemcpyAsync(s->d_dirs, model->dirs, 12 * n, cudaMemcpyHostToDevice, st),
                        "copy dirs");
        if (r == RMG_OK && model->kind == RMG_MODEL_ONDN)
          r = cuda_status(cudaMemcpyAsync(s->d_origs, model->origs, 12 * n, cudaMemcpyHostToDevice, st),
                          "copy origs");
        const std::vector<uint32_t> order = visiting_order(reinterpret_cast<const float*>(model->dirs), n);
        if (r == RMG_OK && !order.empty()) {
          r = dev_alloc(&s->d_order, n, "sensor visiting order");
          if (r == RMG_OK)
            r = cuda_status(cudaMemcpyAsync(s->d_order, order.data(), 4 * n, cudaMemcpyHostToDevice, st),
                            "copy visiting order");
          if (r == RMG_OK) r = cuda_status(cudaStreamSynchronize(st), "sensor sync");  // order is a local
        }
        break;
      }
    }
    if (r == RMG_OK) r = cuda_status(cudaStreamSynchronize(st), "sensor sync");
    if (r != RMG_OK) { free_sensor(s); return r; }
    *out = s;
    return RMG_OK;
  });
}

extern "C" int rmg_sensor_destroy(rmg_sensor* s) {
  return guarded("rmg_sensor_destroy", [&]() -> int {
    free_sensor(s);
    return RMG_OK;
  });
}

extern "C" int rmg_sensor_directions(const rmg_sensor* s, rmg_vec3* host_out) {
  return guarded("rmg_sensor_directions", [&]() -> int {
    if (!s || !host_out) return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_directions: NULL argument");
    RMG_CUDA_TRY(cudaMemcpy(host_out, s->d_dirs, 12ull * s->width * s->height, cudaMemcpyDeviceToHost));
    return RMG_OK;
  });
}

extern "C" int rmg_sensor_visit_order(const rmg_sensor* s, uint32_t* host_out, int* sorted) {
  return guarded("rmg_sensor_visit_order", [&]() -> int {
    if (!s || !sorted) return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_visit_order: NULL argument");
    *sorted = s->d_order ? 1 : 0;
    if (s->d_order && host_out)
      RMG_CUDA_TRY(cudaMemcpy(host_out, s->d_order, 4ull * s->width * s->height, cudaMemcpyDeviceToHost));
    return RMG_OK;
  });
}

extern "C" int rmg_sensor_size(const rmg_sensor* s, uint32_t* width, uint32_t* height) {
  return guarded("rmg_sensor_size", [&]() -> int {
    if (!s) return fail(RMG_ERR_INVALID_ARG, "rmg_sensor_size: sensor is NULL");
    if (width) *width = s->width;
    if (height) *height = s->height;
    return RMG_OK;
  });
}
