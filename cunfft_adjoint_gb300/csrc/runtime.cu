// runtime.cu -- see runtime.h.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <vector>
#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdlib.h>
#include "runtime.h"

namespace cuna {

static thread_local std::string t_last_error;

int fail(int status, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return status;
}

int fail_cuda(cudaError_t e, const char *what) {
  return fail(CUNA2_ERROR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

void clear_error() { t_last_error.clear(); }

// ---------------------------------------------------------------------------
// workspaces
// ---------------------------------------------------------------------------
namespace {
struct Ws {
  void *p = nullptr;
  size_t bytes = 0;
};
std::mutex g_ws_mu;
std::map<std::pair<int, cudaStream_t>, Ws> *g_ws = new std::map<std::pair<int, cudaStream_t>, Ws>();
}  // namespace

int stream_workspace(cudaStream_t stream, size_t bytes, void **ptr) {
  int dev = 0;
  CUNA_CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_ws_mu);
  Ws &w = (*g_ws)[std::make_pair(dev, stream)];
  if (w.bytes < bytes) {
    if (w.p) {
      CUNA_CK(cudaStreamSynchronize(stream));
      CUNA_CK(cudaFree(w.p));
      w.p = nullptr;
      w.bytes = 0;
    }
    size_t want = bytes + bytes / 4 + 4096;
    cudaError_t e = cudaMalloc(&w.p, want);
    if (e != cudaSuccess) {
      w.p = nullptr;
      return fail(CUNA2_ERROR_ALLOC, "workspace allocation of %zu bytes failed: %s", want,
                  cudaGetErrorString(e));
    }
    w.bytes = want;
  }
  *ptr = w.p;
  return CUNA2_SUCCESS;
}

int device_sm_count() {
  static std::mutex mu;
  static std::map<int, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cache[dev] = sms;
  return sms;
}

// ---------------------------------------------------------------------------
// twiddle tables
// ---------------------------------------------------------------------------
namespace {
struct TwEntry {
  FftGeom g;
};
std::mutex g_tw_mu;
std::map<std::tuple<int, int, int>, TwEntry> *g_tw = new std::map<std::tuple<int, int, int>, TwEntry>();

// float-float table entries: the double value as its nearest float and the
// remainder, laid out as the device's float-float complex (re.hi, re.lo,
// im.hi, im.lo)
struct DfPair {
  float hi, lo;
  DfPair() = default;
  explicit DfPair(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

template <typename T>
int upload_table(int64_t count, int64_t step_num, int64_t denom, const void **out) {
  // entries exp(+2 pi i * q * step_num / denom), q < count, in double then rounded
  std::vector<T> h(2 * (size_t)count);
  for (int64_t q = 0; q < count; ++q) {
    // exact reduction of the angle numerator before the trigonometric call
    int64_t num = (q * step_num) % denom;
    double a = 2.0 * M_PI * (double)num / (double)denom;
    h[2 * q] = T(cos(a));
    h[2 * q + 1] = T(sin(a));
  }
  void *d = nullptr;
  size_t bytes = sizeof(T) * h.size();
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(twiddles)");
  e = cudaMemcpy(d, h.data(), bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpy(twiddles)");
  *out = d;
  return CUNA2_SUCCESS;
}
}  // namespace

int fft_geometry_df(int logL, FftGeom *g) {
  if (logL < 2 || logL > kMaxLogL) return fail(CUNA2_ERROR_UNSUPPORTED, "FFT length 2^%d unsupported", logL);
  int dev = 0;
  CUNA_CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto key = std::make_tuple(dev, 4, logL);
  auto it = g_tw->find(key);
  if (it != g_tw->end()) {
    *g = it->second.g;
    return CUNA2_SUCCESS;
  }
  FftGeom G{};
  G.logL = logL;
  G.single = false;
  G.logL1 = (logL + 1) / 2;
  G.logL2 = logL / 2;
  const int64_t L = int64_t(1) << logL, L1 = int64_t(1) << G.logL1, L2 = int64_t(1) << G.logL2;
  const int64_t nlo = L < 2048 ? L : 2048, nhi = L / nlo;
  int st;
  if ((st = upload_table<DfPair>(L1, 1, L1, &G.tw1))) return st;
  if ((st = upload_table<DfPair>(L2, 1, L2, &G.tw2))) return st;
  if ((st = upload_table<DfPair>(nlo, 1, L, &G.twlo))) return st;
  if ((st = upload_table<DfPair>(nhi, nlo, L, &G.twhi))) return st;
  (*g_tw)[key] = TwEntry{G};
  *g = G;
  return CUNA2_SUCCESS;
}

int fft_geometry(bool is_double, int logL, FftGeom *g, bool split) {
  if (logL < 0 || logL > kMaxLogL) return fail(CUNA2_ERROR_UNSUPPORTED, "FFT length 2^%d unsupported", logL);
  int dev = 0;
  CUNA_CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto key = std::make_tuple(dev, (is_double ? 1 : 0) + (split ? 2 : 0), logL);
  auto it = g_tw->find(key);
  if (it != g_tw->end()) {
    *g = it->second.g;
    return CUNA2_SUCCESS;
  }
  FftGeom G{};
  G.logL = logL;
  const int single_log = is_double ? kSingleLogF64 : kSingleLogF32;
  G.single = logL <= single_log && !split;
  if (G.single) {
    G.logL1 = logL;
    G.logL2 = 0;
  } else {
    G.logL1 = (logL + 1) / 2;
    G.logL2 = logL / 2;
  }
  const int64_t L = int64_t(1) << logL, L1 = int64_t(1) << G.logL1, L2 = int64_t(1) << G.logL2;
  const int64_t nlo = L < 2048 ? L : 2048, nhi = L / nlo;
  int st;
  if (is_double) {
    if ((st = upload_table<double>(L1, 1, L1, &G.tw1))) return st;
    if ((st = upload_table<double>(L2, 1, L2, &G.tw2))) return st;
    if ((st = upload_table<double>(nlo, 1, L, &G.twlo))) return st;
    if ((st = upload_table<double>(nhi, nlo, L, &G.twhi))) return st;
  } else {
    if ((st = upload_table<float>(L1, 1, L1, &G.tw1))) return st;
    if ((st = upload_table<float>(L2, 1, L2, &G.tw2))) return st;
    if ((st = upload_table<float>(nlo, 1, L, &G.twlo))) return st;
    if ((st = upload_table<float>(nhi, nlo, L, &G.twhi))) return st;
  }
  (*g_tw)[key] = TwEntry{G};
  *g = G;
  return CUNA2_SUCCESS;
}

}  // namespace cuna

// ---------------------------------------------------------------------------
// extern "C" status helpers
// ---------------------------------------------------------------------------
extern "C" const char *cuna2_last_error(void) { return cuna::t_last_error.c_str(); }

extern "C" const char *cuna2_status_string(int s) {
  switch (s) {
    case CUNA2_SUCCESS: return "CUNA2_SUCCESS";
    case CUNA2_ERROR_INVALID_VALUE: return "CUNA2_ERROR_INVALID_VALUE";
    case CUNA2_ERROR_CUDA: return "CUNA2_ERROR_CUDA";
    case CUNA2_ERROR_UNSUPPORTED: return "CUNA2_ERROR_UNSUPPORTED";
    case CUNA2_ERROR_ALLOC: return "CUNA2_ERROR_ALLOC";
    case CUNA2_ERROR_CUFFT: return "CUNA2_ERROR_CUFFT";
    default: return "CUNA2_ERROR_UNKNOWN";
  }
}

extern "C" const char *cuna2_version(void) { return "cuna-gb300 1.0 (sm_103a)"; }

namespace cuna {
namespace {
int *g_timeouts_host = nullptr;
int *g_timeouts_dev = nullptr;
std::once_flag g_timeouts_once;
}  // namespace

namespace {
std::mutex g_setup_mu;
std::set<std::pair<int, const void *>> *g_setup = new std::set<std::pair<int, const void *>>();
}  // namespace

bool setup_done(const void *key) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  return g_setup->count(std::make_pair(dev, key)) != 0;
}

void mark_setup_done(const void *key) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  g_setup->insert(std::make_pair(dev, key));
}

int *wait_timeout_counter() {
  std::call_once(g_timeouts_once, [] {
    int *h = nullptr, *d = nullptr;
    if (cudaHostAlloc((void **)&h, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    *h = 0;
    if (cudaHostGetDevicePointer((void **)&d, h, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaFreeHost(h);
      return;
    }
    g_timeouts_host = h;
    g_timeouts_dev = d;
  });
  return g_timeouts_dev;
}

namespace {
thread_local bool g_pdl_off = false;
}

void pdl_suppress(bool off) { g_pdl_off = off; }

bool pdl_enabled() {
  static const bool on = [] {
    const char *v = getenv("CUNA2_PDL");
    return !(v && v[0] == '0');
  }();
  return on && !g_pdl_off;
}

bool masked_gather_forced() {
  static const bool on = [] {
    const char *v = getenv("CUNA2_GATHER_MASKS");
    return v && v[0] == '1';
  }();
  return on;
}

bool fp64_passes_forced() {
  static const bool on = [] {
    const char *v = getenv("CUNA2_F64_PASSES");
    return v && v[0] == '1';
  }();
  return on;
}

bool tma_enabled() {
  static const bool on = [] {
    const char *v = getenv("CUNA2_TMA");
    return v && v[0] == '1';
  }();
  return on;
}

bool encode_tmap_f32_3d(void *map, const void *base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t s1,
                        uint64_t s2, uint32_t b0, uint32_t b1) {
  static PFN_cuTensorMapEncodeTiled_v12000 enc = [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }
    return (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }();
  if (!enc) return false;
  const cuuint64_t dims[3] = {d0, d1, d2};
  const cuuint64_t strides[2] = {s1, s2};
  const cuuint32_t box[3] = {b0, b1, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(reinterpret_cast<CUtensorMap *>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base),
             dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace cuna

extern "C" long long cuna2_wait_timeouts(void) {
  cuna::wait_timeout_counter();
  return cuna::g_timeouts_host ? (long long)*(volatile int *)cuna::g_timeouts_host : 0;
}
