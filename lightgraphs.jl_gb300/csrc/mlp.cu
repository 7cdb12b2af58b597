// mlp.cu -- the lgbc_mlp handle of include/lgbc.h: parameters (FP32 master
// copy, BF16 working copy, Adam moments) in device memory, and the host side of
// forward, gradient and training calls.  The arithmetic is in learned.cu.
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "lgbc.h"
#include "lgbc_kernels.h"

using namespace lgbc;

struct lgbc_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float* master = nullptr;        // kMlpParams
  __nv_bfloat16* P = nullptr;     // kMlpParamsPadded
  float* m1 = nullptr;            // Adam first moment
  float* m2 = nullptr;            // Adam second moment
  int64_t t = 0;                  // Adam steps taken
  float mean[4] = {0.f, 0.f, 0.f, 0.f};
  float stdev[4] = {1.f, 1.f, 1.f, 1.f};
  int sms = 0;
  std::mutex mu;
};

namespace {

int fail(int code, const std::string& msg) {
  set_last_error(msg.c_str());
  return code;
}

#define MLP_CUDA(call)                                                             \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(LGBC_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define MLP_TRY(expr)           \
  do {                          \
    int rc_ = (expr);           \
    if (rc_ != LGBC_OK) return rc_; \
  } while (0)

uint64_t splitmix(uint64_t& s) {
  uint64_t x = (s += 0x9E3779B97F4A7C15ull);
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

double uniform01(uint64_t& s) { return static_cast<double>(splitmix(s) >> 11) * 0x1.0p-53; }

MlpNorm norm_of(const lgbc_mlp* m) {
  MlpNorm nm;
  for (int f = 0; f < 4; ++f) {
    nm.mu[f] = m->mean[f];
    nm.isd[f] = 1.0f / m->stdev[f];
  }
  return nm;
}

int check(const lgbc_mlp* m) {
  if (!m) return fail(LGBC_EINVAL, "null MLP handle");
  return LGBC_OK;
}

int use_device(const lgbc_mlp* m) {
  MLP_CUDA(cudaSetDevice(m->device));
  return LGBC_OK;
}

template <class T>
int alloc(T** p, size_t count) {
  *p = nullptr;
  const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T) + 16);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(LGBC_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return LGBC_OK;
}

// Device buffers for one training / gradient call, freed on scope exit.
struct Scratch {
  std::vector<void*> ptrs;
  template <class T>
  int get(T** p, size_t count) {
    MLP_TRY(alloc(p, count));
    ptrs.push_back(*p);
    return LGBC_OK;
  }
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
};

int upload_master(lgbc_mlp* m, const float* host) {
  MLP_CUDA(cudaMemcpyAsync(m->master, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice,
                           m->stream));
  mlp_to_bf16(m->stream, m->master, m->P);
  MLP_CUDA(cudaMemsetAsync(m->m1, 0, sizeof(float) * kMlpParams, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->m2, 0, sizeof(float) * kMlpParams, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  MLP_CUDA(cudaGetLastError());
  m->t = 0;
  return LGBC_OK;
}

int create_impl(lgbc_mlp* m, uint64_t seed) {
  MLP_CUDA(cudaGetDevice(&m->device));
  cudaDeviceProp prop;
  MLP_CUDA(cudaGetDeviceProperties(&prop, m->device));
  m->sms = prop.multiProcessorCount;
  MLP_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  MLP_TRY(alloc(&m->master, kMlpParams));
  MLP_TRY(alloc(&m->P, kMlpParamsPadded));
  MLP_TRY(alloc(&m->m1, kMlpParams));
  MLP_TRY(alloc(&m->m2, kMlpParams));
  if (mlp_configure() != 0) return fail(LGBC_ECUDA, "MLP gradient kernel configuration failed");
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) for every weight and bias
  std::vector<float> w(kMlpParams);
  uint64_t s = seed;
  auto fill = [&](int off, int count, int fan_in) {
    const double b = 1.0 / std::sqrt(static_cast<double>(fan_in));
    for (int i = 0; i < count; ++i) w[off + i] = static_cast<float>((2.0 * uniform01(s) - 1.0) * b);
  };
  fill(kMlpW1, kMlpHidden * 4, 4);
  fill(kMlpB1, kMlpHidden, 4);
  fill(kMlpW2, kMlpHidden * kMlpHidden, kMlpHidden);
  fill(kMlpB2, kMlpHidden, kMlpHidden);
  fill(kMlpW3, kMlpHidden, kMlpHidden);
  fill(kMlpB3, 1, kMlpHidden);
  return upload_master(m, w.data());
}

void destroy_impl(lgbc_mlp* m) {
  if (m->device >= 0) cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->master);
  cudaFree(m->P);
  cudaFree(m->m1);
  cudaFree(m->m2);
  if (m->stream) cudaStreamDestroy(m->stream);
}

}  // namespace

int lgbc::mlp_view(const lgbc_mlp* m, MlpView* out) {
  if (!m) return fail(LGBC_EINVAL, "null MLP handle");
  out->P = m->P;
  out->norm = norm_of(m);
  out->device = m->device;
  return LGBC_OK;
}

extern "C" {

int lgbc_mlp_create(lgbc_mlp** out, uint64_t seed) {
  if (!out) return fail(LGBC_EINVAL, "null output handle");
  *out = nullptr;
  lgbc_mlp* m = new (std::nothrow) lgbc_mlp();
  if (!m) return fail(LGBC_ENOMEM, "host allocation failed");
  const int rc = create_impl(m, seed);
  if (rc != LGBC_OK) {
    destroy_impl(m);
    delete m;
    return rc;
  }
  *out = m;
  return LGBC_OK;
}

int lgbc_mlp_destroy(lgbc_mlp* m) {
  if (!m) return LGBC_OK;
  destroy_impl(m);
  delete m;
  return LGBC_OK;
}

int lgbc_mlp_get_params(const lgbc_mlp* m, float* master, uint16_t* bf16) {
  MLP_TRY(check(m));
  std::lock_guard<std::mutex> lock(const_cast<lgbc_mlp*>(m)->mu);
  MLP_TRY(use_device(m));
  if (master)
    MLP_CUDA(cudaMemcpy(master, m->master, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  if (bf16) MLP_CUDA(cudaMemcpy(bf16, m->P, sizeof(uint16_t) * kMlpParams, cudaMemcpyDeviceToHost));
  return LGBC_OK;
}

int lgbc_mlp_set_params(lgbc_mlp* m, const float* master) {
  MLP_TRY(check(m));
  if (!master) return fail(LGBC_EINVAL, "null parameters");
  for (int i = 0; i < kMlpParams; ++i)
    if (!std::isfinite(master[i])) return fail(LGBC_EINVAL, "non-finite parameter");
  std::lock_guard<std::mutex> lock(m->mu);
  MLP_TRY(use_device(m));
  return upload_master(m, master);
}

int lgbc_mlp_set_norm(lgbc_mlp* m, const float* mean, const float* stdev) {
  MLP_TRY(check(m));
  if (!mean || !stdev) return fail(LGBC_EINVAL, "null standardisation");
  for (int f = 0; f < 4; ++f)
    if (!std::isfinite(mean[f]) || !(stdev[f] > 0.f) || !std::isfinite(stdev[f]))
      return fail(LGBC_EINVAL, "standard deviations must be finite and positive");
  std::lock_guard<std::mutex> lock(m->mu);
  std::memcpy(m->mean, mean, sizeof(m->mean));
  std::memcpy(m->stdev, stdev, sizeof(m->stdev));
  return LGBC_OK;
}

int lgbc_mlp_get_norm(const lgbc_mlp* m, float* mean, float* stdev) {
  MLP_TRY(check(m));
  if (mean) std::memcpy(mean, m->mean, sizeof(m->mean));
  if (stdev) std::memcpy(stdev, m->stdev, sizeof(m->stdev));
  return LGBC_OK;
}

int lgbc_mlp_forward(lgbc_mlp* m, const float* x, int64_t rows, float* y) {
  MLP_TRY(check(m));
  if (rows < 0 || (rows > 0 && (!x || !y))) return fail(LGBC_EINVAL, "bad rows or null buffer");
  std::lock_guard<std::mutex> lock(m->mu);
  MLP_TRY(use_device(m));
  if (rows == 0) return LGBC_OK;
  Scratch sc;
  float4* dx;
  float* dy;
  MLP_TRY(sc.get(&dx, static_cast<size_t>(rows)));
  MLP_TRY(sc.get(&dy, static_cast<size_t>(rows)));
  MLP_CUDA(cudaMemcpyAsync(dx, x, sizeof(float4) * rows, cudaMemcpyHostToDevice, m->stream));
  const LaunchCfg c{m->sms * 8, 256, m->sms};
  mlp_forward(c, m->stream, dx, rows, m->P, norm_of(m), dy);
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpyAsync(y, dy, sizeof(float) * rows, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return LGBC_OK;
}

int lgbc_mlp_grad(lgbc_mlp* m, const float* x, const float* target, int64_t rows, float* grad,
                  float* loss) {
  MLP_TRY(check(m));
  if (rows <= 0 || rows > (1 << 24) || !x || !target || !grad)
    return fail(LGBC_EINVAL, "rows must be in [1, 2^24] and buffers non-null");
  std::lock_guard<std::mutex> lock(m->mu);
  MLP_TRY(use_device(m));
  const int B = static_cast<int>(rows);
  const int nb = (B + kGradRows - 1) / kGradRows;
  Scratch sc;
  float4* dx;
  float *dt, *de, *dcenter, *dpart, *dloss, *dgrad;
  MLP_TRY(sc.get(&dx, static_cast<size_t>(B)));
  MLP_TRY(sc.get(&dt, static_cast<size_t>(B)));
  MLP_TRY(sc.get(&de, static_cast<size_t>(B)));
  MLP_TRY(sc.get(&dcenter, 1));
  MLP_TRY(sc.get(&dpart, static_cast<size_t>(nb) * kMlpParams));
  MLP_TRY(sc.get(&dloss, 1));
  MLP_TRY(sc.get(&dgrad, kMlpParams));
  MLP_CUDA(cudaMemcpyAsync(dx, x, sizeof(float4) * B, cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaMemcpyAsync(dt, target, sizeof(float) * B, cudaMemcpyHostToDevice, m->stream));
  mlp_train_step(m->stream, dx, dt, 0, B, m->P, norm_of(m), de, dcenter, dpart, dloss, dgrad, nullptr,
                 nullptr, nullptr, nullptr, AdamStep{});
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpyAsync(grad, dgrad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost,
                           m->stream));
  float l = 0.f;
  MLP_CUDA(cudaMemcpyAsync(&l, dloss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  if (loss) *loss = l;
  return LGBC_OK;
}

int lgbc_mlp_train(lgbc_mlp* m, const float* x, const float* target, int64_t rows,
                   const int64_t* group_off, int64_t ngroups, const lgbc_train_cfg* cfg,
                   float* loss_out) {
  MLP_TRY(check(m));
  if (!cfg || !x || !target || !group_off || rows <= 0 || ngroups <= 0)
    return fail(LGBC_EINVAL, "null argument or empty training set");
  if (cfg->steps < 0 || cfg->batch < 2 || cfg->batch > (1 << 20) || cfg->warmup < 0 ||
      !(cfg->lr >= 0.f) || !(cfg->lr_final >= 0.f) || !(cfg->beta1 >= 0.f && cfg->beta1 < 1.f) ||
      !(cfg->beta2 >= 0.f && cfg->beta2 < 1.f) || !(cfg->eps > 0.f))
    return fail(LGBC_EINVAL, "bad training configuration");
  if (group_off[0] != 0 || group_off[ngroups] != rows)
    return fail(LGBC_EINVAL, "group offsets must run from 0 to rows");
  for (int64_t gi = 0; gi < ngroups; ++gi)
    if (group_off[gi + 1] - group_off[gi] < 2) return fail(LGBC_EINVAL, "every group needs 2 rows");
  std::lock_guard<std::mutex> lock(m->mu);
  MLP_TRY(use_device(m));
  const int Bmax = cfg->batch;
  const int nb = (Bmax + kGradRows - 1) / kGradRows;
  Scratch sc;
  float4* dx;
  float *dt, *de, *dcenter, *dpart, *dloss;
  MLP_TRY(sc.get(&dx, static_cast<size_t>(rows)));
  MLP_TRY(sc.get(&dt, static_cast<size_t>(rows)));
  MLP_TRY(sc.get(&de, static_cast<size_t>(Bmax)));
  MLP_TRY(sc.get(&dcenter, 1));
  MLP_TRY(sc.get(&dpart, static_cast<size_t>(nb) * kMlpParams));
  MLP_TRY(sc.get(&dloss, static_cast<size_t>(cfg->steps > 0 ? cfg->steps : 1)));
  MLP_CUDA(cudaMemcpyAsync(dx, x, sizeof(float4) * rows, cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaMemcpyAsync(dt, target, sizeof(float) * rows, cudaMemcpyHostToDevice, m->stream));
  const MlpNorm nm = norm_of(m);
  uint64_t rs = cfg->seed;
  const double pi = 3.14159265358979323846;
  for (int32_t step = 0; step < cfg->steps; ++step) {
    const int64_t gi = static_cast<int64_t>(uniform01(rs) * static_cast<double>(ngroups));
    const int64_t g0 = group_off[gi], gn = group_off[gi + 1] - g0;
    const int B = static_cast<int>(gn < Bmax ? gn : Bmax);
    const int64_t r0 = g0 + static_cast<int64_t>(uniform01(rs) * static_cast<double>(gn - B + 1));
    double lr;
    if (step < cfg->warmup) {
      lr = cfg->lr * static_cast<double>(step + 1) / static_cast<double>(cfg->warmup);
    } else {
      const int span = cfg->steps - cfg->warmup;
      const double frac = span > 1 ? static_cast<double>(step - cfg->warmup) / (span - 1) : 1.0;
      lr = cfg->lr_final + 0.5 * (cfg->lr - cfg->lr_final) * (1.0 + std::cos(pi * frac));
    }
    m->t += 1;
    AdamStep st;
    st.lr = static_cast<float>(lr);
    st.beta1 = cfg->beta1;
    st.beta2 = cfg->beta2;
    st.eps = cfg->eps;
    st.bc1 = static_cast<float>(1.0 - std::pow(static_cast<double>(cfg->beta1), static_cast<double>(m->t)));
    st.bc2 = static_cast<float>(1.0 - std::pow(static_cast<double>(cfg->beta2), static_cast<double>(m->t)));
    mlp_train_step(m->stream, dx, dt, r0, B, m->P, nm, de, dcenter, dpart, dloss + step, nullptr,
                   m->master,
                   m->P, m->m1, m->m2, st);
  }
  MLP_CUDA(cudaGetLastError());
  if (loss_out && cfg->steps > 0)
    MLP_CUDA(cudaMemcpyAsync(loss_out, dloss, sizeof(float) * cfg->steps, cudaMemcpyDeviceToHost,
                             m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return LGBC_OK;
}

}  // extern "C"
