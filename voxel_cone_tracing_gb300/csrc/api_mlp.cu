// api_mlp.cu -- C ABI of the learned diffuse term (include/vct.h): network
// allocation and seeded initialisation, training-data generation on the
// scene of the last frame, the Adam training loop, checkpoints, and the
// evaluation / gradient hooks the tests use.
#include <cstdio>
#include <cstring>

#include "renderer_state.h"

namespace {

constexpr uint32_t kMagic = 0x504c4d56u;  // "VMLP"
constexpr uint32_t kVersion = 1;

struct CkptHeader {
  uint32_t magic, version;
  int32_t levels, log2_table, n_min, n_max;
  int32_t adam_t;
  uint32_t reserved[9];
};

vct_status check_desc(const vct_mlp_desc& d) {
  if (d.levels != kMlpLevels) return set_error(VCT_ERR_INVALID_VALUE, "levels must be %d", kMlpLevels);
  if (d.log2_table < 8 || d.log2_table > 24) return set_error(VCT_ERR_INVALID_VALUE, "log2_table %d", d.log2_table);
  if (d.n_min < 2 || d.n_max < d.n_min || d.n_max > 1 << 16)
    return set_error(VCT_ERR_INVALID_VALUE, "resolutions %d..%d", d.n_min, d.n_max);
  return VCT_OK;
}

vct_status alloc_and_init(vct_renderer* r, const vct_mlp_desc& d) {
  VCT_CHECK(check_desc(d));
  MlpState& m = r->mlp;
  m.levels = d.levels;
  m.log2_table = d.log2_table;
  m.n_min = d.n_min;
  m.n_max = d.n_max;
  const size_t tf = m.table_floats();
  VCT_CHECK(m.table.ensure(tf));
  VCT_CHECK(m.table_grad.ensure(tf));
  VCT_CHECK(m.table_m.ensure(tf));
  VCT_CHECK(m.table_v.ensure(tf));
  VCT_CHECK(m.table_bf.ensure(tf));
  VCT_CHECK(m.w.ensure(kMlpWeights));
  VCT_CHECK(m.w_grad.ensure(kMlpWeights));
  VCT_CHECK(m.w_m.ensure(kMlpWeights));
  VCT_CHECK(m.w_v.ensure(kMlpWeights));
  VCT_CHECK(m.w_bf.ensure(kMlpWeights));
  cudaStream_t st = r->stream;
  VCT_CUDA(launch_mlp_init(m.table.p, m.table_bf.p, tf, 1e-4f, d.seed * 2 + 1, st));
  // He-uniform for the ReLU layers; W5 rows 3..15 stay zero (unused outputs).
  VCT_CUDA(launch_mlp_init(m.w.p, m.w_bf.p, 4 * 4096, std::sqrt(6.0f / 64.0f), d.seed * 2 + 2, st));
  VCT_CUDA(launch_mlp_init(m.w.p + 4 * 4096, m.w_bf.p + 4 * 4096, 3 * 64, std::sqrt(6.0f / 64.0f), d.seed * 2 + 3,
                           st));
  VCT_CUDA(cudaMemsetAsync(m.w.p + 4 * 4096 + 3 * 64, 0, (kMlpWeights - 4 * 4096 - 3 * 64) * sizeof(float), st));
  VCT_CUDA(cudaMemsetAsync(m.w_bf.p + 4 * 4096 + 3 * 64, 0,
                           (kMlpWeights - 4 * 4096 - 3 * 64) * sizeof(__nv_bfloat16), st));
  for (DevBuf<float>* b : {&m.table_grad, &m.table_m, &m.table_v})
    VCT_CUDA(cudaMemsetAsync(b->p, 0, tf * sizeof(float), st));
  for (DevBuf<float>* b : {&m.w_grad, &m.w_m, &m.w_v}) VCT_CUDA(cudaMemsetAsync(b->p, 0, kMlpWeights * sizeof(float), st));
  VCT_CUDA(cudaStreamSynchronize(st));
  m.adam_t = 0;
  m.ready = true;
  m.trained = false;
  return VCT_OK;
}

// Copy host rows into the sample buffer.
vct_status upload_samples(vct_renderer* r, const float* rows, uint32_t n) {
  VCT_CHECK(r->mlp.samples.ensure((size_t)n * 12));
  VCT_CUDA(cudaMemcpyAsync(r->mlp.samples.p, rows, (size_t)n * 12 * sizeof(float), cudaMemcpyHostToDevice, r->stream));
  r->mlp.n_samples = n;
  return VCT_OK;
}

// Adam on both parameter groups (instant-NGP style hyper-parameters:
// beta1 0.9, beta2 0.99, eps 1e-15; 1e-6 L2 on the MLP weights).
vct_status adam_step(vct_renderer* r, float lr) {
  MlpState& m = r->mlp;
  ++m.adam_t;
  AdamStep a;
  a.lr = lr;
  a.beta1 = 0.9f;
  a.beta2 = 0.99f;
  a.eps = 1e-15f;
  a.c1 = (float)(1.0 / (1.0 - std::pow(0.9, m.adam_t)));
  a.c2 = (float)(1.0 / (1.0 - std::pow(0.99, m.adam_t)));
  a.l2 = 1e-6f;
  VCT_CUDA(launch_adam(m.w.p, m.w_grad.p, m.w_m.p, m.w_v.p, m.w_bf.p, kMlpWeights, a, r->stream));
  a.l2 = 0.0f;
  VCT_CUDA(launch_adam(m.table.p, m.table_grad.p, m.table_m.p, m.table_v.p, m.table_bf.p, m.table_floats(), a,
                       r->stream));
  return VCT_OK;
}

vct_status train_loop(vct_renderer* r, const vct_mlp_desc& d, vct_mlp_report* rep, float ms_samples) {
  MlpState& m = r->mlp;
  if (!m.n_samples) return set_error(VCT_ERR_INVALID_VALUE, "no training samples");
  const uint32_t steps = d.steps ? d.steps : 1;
  const uint32_t batch = std::max<uint32_t>(16, std::min(d.batch ? d.batch : (1u << 18), m.n_samples));
  VCT_CHECK(m.loss.ensure(steps));
  VCT_CUDA(cudaMemsetAsync(m.loss.p, 0, steps * sizeof(float), r->stream));
  const MlpParams p = m.params();
  cudaEvent_t e0, e1;
  VCT_CUDA(cudaEventCreate(&e0));
  VCT_CUDA(cudaEventCreate(&e1));
  VCT_CUDA(cudaEventRecord(e0, r->stream));
  for (uint32_t s = 0; s < steps; ++s) {
    MlpBatch b;
    b.samples = m.samples.p;
    b.total = (int)m.n_samples;
    b.first = (int)(((uint64_t)s * batch) % m.n_samples);
    b.n = (int)batch;
    VCT_CUDA(launch_mlp_train(p, b, m.loss.p + s, r->stream));
    // Constant for the first half of the steps, then decaying geometrically
    // to a tenth (the optimiser settles instead of ending on a noisy step).
    const double t = steps > 1 ? std::max(0.0, ((double)s - 0.5 * steps) / (0.5 * steps)) : 0.0;
    VCT_CHECK(adam_step(r, (float)(d.lr * std::pow(0.1, t))));
  }
  VCT_CUDA(cudaEventRecord(e1, r->stream));
  VCT_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::vector<float> loss(steps);
  VCT_CUDA(cudaMemcpy(loss.data(), m.loss.p, steps * sizeof(float), cudaMemcpyDeviceToHost));
  m.trained = true;
  if (rep) {
    rep->loss_first = loss[0];
    const uint32_t tail = std::max<uint32_t>(1, steps / 10);
    double acc = 0.0;
    for (uint32_t s = steps - tail; s < steps; ++s) acc += loss[s];
    rep->loss_last = (float)(acc / tail);
    rep->ms_samples = ms_samples;
    rep->ms_train = ms;
    rep->steps = steps;
    rep->n_samples = m.n_samples;
  }
  return VCT_OK;
}

}  // namespace

extern "C" void vct_mlp_desc_default(vct_mlp_desc* d) {
  if (!d) return;
  std::memset(d, 0, sizeof(*d));
  d->levels = 16;
  d->log2_table = 19;
  d->n_min = 16;
  d->n_max = 512;
  d->n_samples = 1u << 24;
  d->batch = 1u << 18;
  d->steps = 1000;
  d->lr = 1e-2f;
  d->seed = 1;
}

extern "C" vct_status vct_mlp_init(vct_renderer* r, const vct_mlp_desc* d) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  vct_mlp_desc dd;
  if (d) dd = *d; else vct_mlp_desc_default(&dd);
  VCT_CHECK(r->finish());
  return alloc_and_init(r, dd);
}

extern "C" vct_status vct_mlp_train(vct_renderer* r, const vct_mlp_desc* d, vct_mlp_report* report) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  vct_mlp_desc dd;
  if (d) dd = *d; else vct_mlp_desc_default(&dd);
  VCT_CHECK(r->finish());
  if (!r->have_sp || !r->last_sp.total_tris)
    return set_error(VCT_ERR_INVALID_VALUE, "render a frame with queued models before training");
  if (!dd.n_samples) return set_error(VCT_ERR_INVALID_VALUE, "n_samples is 0");
  VCT_CHECK(alloc_and_init(r, dd));
  MlpState& m = r->mlp;
  const SceneParams& sp = r->last_sp;
  cudaStream_t st = r->stream;
  cudaEvent_t e0, e1;
  VCT_CUDA(cudaEventCreate(&e0));
  VCT_CUDA(cudaEventCreate(&e1));
  VCT_CUDA(cudaEventRecord(e0, st));
  // Area CDF of the queued triangles (prefix sums in double on the host).
  DevBuf<float> area;
  VCT_CHECK(area.ensure(sp.total_tris));
  VCT_CUDA(launch_tri_area(sp, area.p, st));
  std::vector<float> a(sp.total_tris);
  VCT_CUDA(cudaMemcpyAsync(a.data(), area.p, sp.total_tris * sizeof(float), cudaMemcpyDeviceToHost, st));
  VCT_CUDA(cudaStreamSynchronize(st));
  double run = 0.0;
  for (auto& v : a) {
    run += v;
    v = (float)run;
  }
  if (!(run > 0.0)) return set_error(VCT_ERR_INVALID_VALUE, "queued triangles have zero total area");
  VCT_CUDA(cudaMemcpyAsync(area.p, a.data(), sp.total_tris * sizeof(float), cudaMemcpyHostToDevice, st));
  VCT_CHECK(m.samples.ensure((size_t)dd.n_samples * 12));
  m.n_samples = dd.n_samples;
  VCT_CUDA(launch_sample_surface(sp, area.p, (int)dd.n_samples, dd.seed, m.samples.p, st));
  VCT_CUDA(launch_trace_points(sp, r->ms, r->cfg.mip_mode, r->cfg.cone_set, m.samples.p, (int)dd.n_samples, st));
  VCT_CUDA(cudaEventRecord(e1, st));
  VCT_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return train_loop(r, dd, report, ms);
}

extern "C" vct_status vct_mlp_train_samples(vct_renderer* r, const float* samples, uint32_t n, const vct_mlp_desc* d,
                                            vct_mlp_report* report) {
  clear_error();
  if (!r || !samples || !n) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer / samples or n = 0");
  vct_mlp_desc dd;
  if (d) dd = *d; else vct_mlp_desc_default(&dd);
  VCT_CHECK(r->finish());
  if (!r->mlp.ready) VCT_CHECK(alloc_and_init(r, dd));
  VCT_CHECK(upload_samples(r, samples, n));
  return train_loop(r, dd, report, 0.0f);
}

extern "C" vct_status vct_set_diffuse_mode(vct_renderer* r, int32_t mode) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (mode != VCT_DIFFUSE_CONES && mode != VCT_DIFFUSE_MLP)
    return set_error(VCT_ERR_INVALID_VALUE, "diffuse mode %d", mode);
  if (mode == VCT_DIFFUSE_MLP && !r->mlp.trained)
    return set_error(VCT_ERR_INVALID_VALUE, "the learned diffuse term is not trained (vct_mlp_train / vct_mlp_load)");
  r->diffuse_mode = mode;
  return VCT_OK;
}

extern "C" vct_status vct_mlp_set_judge(vct_renderer* r, int32_t stride, float min_psnr_db) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (stride < 0 || stride > 256) return set_error(VCT_ERR_INVALID_VALUE, "judge stride %d (0 = off, 1..256)", stride);
  if (!(min_psnr_db >= 0.0f) || !(min_psnr_db < 200.0f))
    return set_error(VCT_ERR_INVALID_VALUE, "judge threshold %g dB", (double)min_psnr_db);
  VCT_CHECK(r->finish());
  r->judge_stride = stride;
  r->judge_min_psnr = min_psnr_db;
  return VCT_OK;
}

extern "C" vct_status vct_mlp_get_judge(vct_renderer* r, vct_mlp_judge_report* out) {
  clear_error();
  if (!r || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  VCT_CHECK(r->finish());
  std::memset(out, 0, sizeof(*out));
  out->last_psnr_db = r->judge_last_psnr;
  out->judged_pixels = r->judge_last_n;
  out->fallbacks = r->judge_fallbacks;
  out->diffuse_mode = r->diffuse_mode;
  out->stride = r->judge_stride;
  out->min_psnr_db = r->judge_min_psnr;
  return VCT_OK;
}

extern "C" vct_status vct_mlp_get_params(vct_renderer* r, float* table, float* weights) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (!r->mlp.ready) return set_error(VCT_ERR_INVALID_VALUE, "network not initialised");
  VCT_CHECK(r->finish());
  if (table) VCT_CUDA(cudaMemcpy(table, r->mlp.table.p, r->mlp.table_floats() * sizeof(float), cudaMemcpyDeviceToHost));
  if (weights) VCT_CUDA(cudaMemcpy(weights, r->mlp.w.p, kMlpWeights * sizeof(float), cudaMemcpyDeviceToHost));
  return VCT_OK;
}

namespace {
__global__ void k_to_bf16(const float* __restrict__ a, __nv_bfloat16* __restrict__ b, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}
vct_status refresh_bf16(vct_renderer* r) {
  MlpState& m = r->mlp;
  k_to_bf16<<<1024, 256, 0, r->stream>>>(m.table.p, m.table_bf.p, m.table_floats());
  k_to_bf16<<<64, 256, 0, r->stream>>>(m.w.p, m.w_bf.p, kMlpWeights);
  VCT_CUDA(cudaGetLastError());
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  return VCT_OK;
}
}  // namespace

extern "C" vct_status vct_mlp_set_params(vct_renderer* r, const float* table, const float* weights) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  if (!r->mlp.ready) return set_error(VCT_ERR_INVALID_VALUE, "network not initialised");
  VCT_CHECK(r->finish());
  if (table) VCT_CUDA(cudaMemcpy(r->mlp.table.p, table, r->mlp.table_floats() * sizeof(float), cudaMemcpyHostToDevice));
  if (weights) VCT_CUDA(cudaMemcpy(r->mlp.w.p, weights, kMlpWeights * sizeof(float), cudaMemcpyHostToDevice));
  return refresh_bf16(r);
}

extern "C" vct_status vct_mlp_eval(vct_renderer* r, const float* samples, uint32_t n, float* rgb_out) {
  clear_error();
  if (!r || !samples || !rgb_out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (!r->mlp.ready) return set_error(VCT_ERR_INVALID_VALUE, "network not initialised");
  if (!n) return VCT_OK;
  VCT_CHECK(r->finish());
  DevBuf<float> in, out;
  VCT_CHECK(in.ensure((size_t)n * 12));
  VCT_CHECK(out.ensure((size_t)n * 3));
  VCT_CUDA(cudaMemcpyAsync(in.p, samples, (size_t)n * 12 * sizeof(float), cudaMemcpyHostToDevice, r->stream));
  DevBuf<FrameStatus> st;
  VCT_CHECK(st.ensure(1));
  VCT_CUDA(cudaMemsetAsync(st.p, 0, sizeof(FrameStatus), r->stream));
  VCT_CUDA(launch_mlp_eval(r->mlp.params(), in.p, (int)n, out.p, r->stream, r->mlp.tc, st.p));
  VCT_CUDA(cudaMemcpyAsync(rgb_out, out.p, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost, r->stream));
  FrameStatus hs;
  VCT_CUDA(cudaMemcpyAsync(&hs, st.p, sizeof(FrameStatus), cudaMemcpyDeviceToHost, r->stream));
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  if (hs.async_timeout) return set_error(VCT_ERR_CUDA, "a tensor-core group did not complete");
  return VCT_OK;
}

extern "C" vct_status vct_mlp_gradients(vct_renderer* r, const float* samples, uint32_t n, float* loss,
                                        float* dweights, float* dtable) {
  clear_error();
  if (!r || !samples || !n) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument or n = 0");
  if (!r->mlp.ready) return set_error(VCT_ERR_INVALID_VALUE, "network not initialised");
  VCT_CHECK(r->finish());
  MlpState& m = r->mlp;
  DevBuf<float> in, l;
  VCT_CHECK(in.ensure((size_t)n * 12));
  VCT_CHECK(l.ensure(1));
  VCT_CUDA(cudaMemcpyAsync(in.p, samples, (size_t)n * 12 * sizeof(float), cudaMemcpyHostToDevice, r->stream));
  VCT_CUDA(cudaMemsetAsync(l.p, 0, sizeof(float), r->stream));
  VCT_CUDA(cudaMemsetAsync(m.w_grad.p, 0, kMlpWeights * sizeof(float), r->stream));
  VCT_CUDA(cudaMemsetAsync(m.table_grad.p, 0, m.table_floats() * sizeof(float), r->stream));
  MlpBatch b;
  b.samples = in.p;
  b.first = 0;
  b.n = (int)n;
  b.total = (int)n;
  VCT_CUDA(launch_mlp_train(m.params(), b, l.p, r->stream));
  if (loss) VCT_CUDA(cudaMemcpyAsync(loss, l.p, sizeof(float), cudaMemcpyDeviceToHost, r->stream));
  if (dweights)
    VCT_CUDA(cudaMemcpyAsync(dweights, m.w_grad.p, kMlpWeights * sizeof(float), cudaMemcpyDeviceToHost, r->stream));
  if (dtable)
    VCT_CUDA(cudaMemcpyAsync(dtable, m.table_grad.p, m.table_floats() * sizeof(float), cudaMemcpyDeviceToHost,
                             r->stream));
  VCT_CUDA(cudaMemsetAsync(m.w_grad.p, 0, kMlpWeights * sizeof(float), r->stream));
  VCT_CUDA(cudaMemsetAsync(m.table_grad.p, 0, m.table_floats() * sizeof(float), r->stream));
  VCT_CUDA(cudaStreamSynchronize(r->stream));
  return VCT_OK;
}

extern "C" vct_status vct_mlp_save(vct_renderer* r, const char* path) {
  clear_error();
  if (!r || !path) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (!r->mlp.ready) return set_error(VCT_ERR_INVALID_VALUE, "network not initialised");
  VCT_CHECK(r->finish());
  MlpState& m = r->mlp;
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  h.magic = kMagic;
  h.version = kVersion;
  h.levels = m.levels;
  h.log2_table = m.log2_table;
  h.n_min = m.n_min;
  h.n_max = m.n_max;
  h.adam_t = m.adam_t;
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(VCT_ERR_IO, "cannot write %s", path);
  std::vector<float> buf(std::max<size_t>(m.table_floats(), kMlpWeights));
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
  for (DevBuf<float>* b : {&m.table, &m.table_m, &m.table_v}) {
    if (cudaMemcpy(buf.data(), b->p, m.table_floats() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
    ok = ok && std::fwrite(buf.data(), sizeof(float), m.table_floats(), f) == m.table_floats();
  }
  for (DevBuf<float>* b : {&m.w, &m.w_m, &m.w_v}) {
    if (cudaMemcpy(buf.data(), b->p, kMlpWeights * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
    ok = ok && std::fwrite(buf.data(), sizeof(float), kMlpWeights, f) == (size_t)kMlpWeights;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return set_error(VCT_ERR_IO, "writing %s failed", path);
  return VCT_OK;
}

extern "C" vct_status vct_mlp_load(vct_renderer* r, const char* path) {
  clear_error();
  if (!r || !path) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  VCT_CHECK(r->finish());
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(VCT_ERR_IO, "cannot read %s", path);
  CkptHeader h;
  if (std::fread(&h, sizeof(h), 1, f) != 1 || h.magic != kMagic) {
    std::fclose(f);
    return set_error(VCT_ERR_IO, "%s is not a network checkpoint", path);
  }
  if (h.version != kVersion) {
    std::fclose(f);
    return set_error(VCT_ERR_IO, "%s: checkpoint version %u, expected %u", path, h.version, kVersion);
  }
  vct_mlp_desc d;
  vct_mlp_desc_default(&d);
  d.levels = h.levels;
  d.log2_table = h.log2_table;
  d.n_min = h.n_min;
  d.n_max = h.n_max;
  vct_status s = alloc_and_init(r, d);
  if (s != VCT_OK) {
    std::fclose(f);
    return s;
  }
  MlpState& m = r->mlp;
  std::vector<float> buf(std::max<size_t>(m.table_floats(), kMlpWeights));
  bool ok = true;
  for (DevBuf<float>* b : {&m.table, &m.table_m, &m.table_v}) {
    ok = ok && std::fread(buf.data(), sizeof(float), m.table_floats(), f) == m.table_floats();
    if (ok && cudaMemcpy(b->p, buf.data(), m.table_floats() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
      ok = false;
  }
  for (DevBuf<float>* b : {&m.w, &m.w_m, &m.w_v}) {
    ok = ok && std::fread(buf.data(), sizeof(float), kMlpWeights, f) == (size_t)kMlpWeights;
    if (ok && cudaMemcpy(b->p, buf.data(), kMlpWeights * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) ok = false;
  }
  std::fclose(f);
  if (!ok) return set_error(VCT_ERR_IO, "%s is truncated", path);
  m.adam_t = h.adam_t;
  VCT_CHECK(refresh_bf16(r));
  m.trained = true;
  return VCT_OK;
}

extern "C" vct_status vct_mlp_set_tensor_kernels(vct_renderer* r, int32_t use_tcgen05) {
  clear_error();
  if (!r) return set_error(VCT_ERR_INVALID_VALUE, "NULL renderer");
  VCT_CHECK(r->finish());
  r->mlp.tc = use_tcgen05 != 0;
  return VCT_OK;
}
