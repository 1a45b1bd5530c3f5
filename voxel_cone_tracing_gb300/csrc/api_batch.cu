// api_batch.cu -- batched rendering: many independent scenes per frame, each
// stage pass one persistent launch over all of them, optionally captured
// once in a CUDA graph and replayed.
//
// Layout.  Every scene keeps its own voxel maps (MapStore) and geometry; the
// per-frame work arrays are batch-wide and each scene uses a slice:
//   bricks      -- scene s owns bricks [brick_base, brick_base + (N/8)^3) of
//                  the count / offset / cursor arrays; one exclusive scan
//                  over all of them gives global positions in one pair list;
//   pixels      -- scene s owns pixels [px_base, px_base + W*H) of the
//                  visibility buffer, the G-buffer and the frame;
//   work items  -- prefix tables map a global item (triangle, brick, mip
//                  region, texel, tile) to its scene.  Triangle ranges are
//                  padded to multiples of 32 so that a warp bins one scene.
// Capacity overflow of the pair list or the record lists is detected on the
// device (FrameStatus), the lists grown and the frame encoded again, exactly
// as a Renderer does; growing invalidates a captured graph, which is then
// captured again on the next frame.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "renderer_state.h"

namespace {

int device_sms() {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

struct SceneRes {
  int W = 0, H = 0, N = 0, L = 0;
  uint32_t n_tris = 0;
  MapStore maps;
  std::vector<std::unique_ptr<DevBuf<vct_vert_data>>> verts;
  std::vector<std::unique_ptr<DevBuf<uint32_t>>> indices, tri_mat;
  DevBuf<DevInstance> inst;
  DevBuf<vct_material_data> materials;
  DevBuf<uint32_t> identity;  // draw object (= material) -> material
  SceneParams sp;
  TraceParams tp;
  float view[16], proj[16];
};

// Host prefix of per-scene item counts (+ device copy).
struct Prefix {
  std::vector<uint32_t> h;
  DevBuf<uint32_t> d;
  uint32_t total() const { return h.empty() ? 0 : h.back(); }
};

}  // namespace

struct vct_batch {
  vct_batch_config cfg;
  std::vector<std::unique_ptr<SceneRes>> scenes;
  int sms = 148;
  BatchShape shape = {8, 8, 3, 1, 1, 16};  // (16-row trace tiles, as a Renderer's)
  // device descriptors
  DevBuf<BatchScene> d_scenes;
  HostBuf<CameraParams> h_cams;
  DevBuf<CameraParams> d_cams;
  Prefix tris, bricks, regions, tail4, tail5, tail6, tiles, occw;
  // The brick kernel writes mip levels 1-3 (per-scene targets in d_mips);
  // the mip pass then runs the tail levels from level 4.
  bool fused = false;
  DevBuf<BrickMips> d_mips;
  std::vector<uint32_t> brick_base;
  std::vector<size_t> px_base;
  size_t total_px = 0;
  // batch-wide work arrays
  DevBuf<uint32_t> brick_count, brick_offset, brick_cursor, pair_list, scan_tmp, bin_big_count, queue;
  DevBuf<uint8_t> brick_dirty;  // BatchBuffers::dirty
  DevBuf<BinRec> bin_big;
  DevBuf<uint2> bin_rec;  // per padded batch triangle (counting -> filling pass)
  uint32_t bin_big_cap = 0;
  HeavyStore heavy;
  DevBuf<unsigned char> rbig;
  DevBuf<uint32_t> rbig_count, rbig_offset;
  uint32_t rbig_cap = 0;
  DevBuf<unsigned long long> vis;
  DevBuf<float4> gb_pos, gb_nrm;
  DevBuf<uchar4> frame;
  DevBuf<FrameStatus> d_status;
  HostBuf<FrameStatus> h_status;
  // execution
  cudaStream_t own_stream = nullptr, stream = nullptr;
  static constexpr int kSide = 4;  // parallel streams of the per-scene trace
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kSide] = {};
  std::vector<int> trace_order;    // scenes, largest frame first
  cudaEvent_t ev[5] = {};
  cudaGraphExec_t graph = nullptr;
  bool pending = false, have_frame = false;
  int launches = 0;

  ~vct_batch() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graph();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (int k = 0; k < kSide; ++k) {
      if (join_ev[k]) cudaEventDestroy(join_ev[k]);
      if (side[k]) cudaStreamDestroy(side[k]);
    }
    if (own_stream) cudaStreamDestroy(own_stream);
  }

  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
  }

  BatchBuffers buffers() const {
    BatchBuffers bb;
    std::memset(&bb, 0, sizeof(bb));
    bb.brick_count = brick_count.p;
    bb.brick_offset = brick_offset.p;
    bb.brick_cursor = brick_cursor.p;
    bb.pair_list = pair_list.p;
    bb.pair_cap = (uint32_t)pair_list.n;
    bb.big = bin_big.p;
    bb.big_cap = bin_big_cap;
    bb.big_count = bin_big_count.p;
    bb.status = d_status.p;
    bb.rb.vis = vis.p;
    bb.rb.big = rbig.p;
    bb.rb.big_cap = rbig_cap;
    bb.rb.big_count = rbig_count.p;
    bb.rb.big_offset = rbig_offset.p;
    bb.rb.scan_tmp = nullptr;
    bb.rb.gb_pos = gb_pos.p;
    bb.rb.gb_nrm = gb_nrm.p;
    bb.rb.status = d_status.p;
    bb.frame = frame.p;
    bb.heavy = kHeavySplit ? heavy.view() : HeavyBricks{};
    bb.bin_rec = bin_rec.p;
    bb.dirty = brick_dirty.p;
    bb.mips = fused ? d_mips.p : nullptr;
    return bb;
  }

  BatchWork work(const Prefix& p, bool with_queue = false) const {
    BatchWork w;
    w.scenes = d_scenes.p;
    w.cams = d_cams.p;
    w.n = (int)scenes.size();
    w.prefix = p.d.p;
    w.total = p.total();
    w.queue = with_queue ? queue.p : nullptr;
    return w;
  }

  vct_status grow_bin_big(uint32_t cap) {
    VCT_CHECK(bin_big.ensure(cap));
    bin_big_cap = cap;
    return VCT_OK;
  }
  vct_status grow_rbig(uint32_t cap) {
    VCT_CHECK(rbig.ensure((size_t)cap * big_record_bytes()));
    VCT_CHECK(rbig_offset.ensure((size_t)cap + 1));
    rbig_cap = cap;
    return VCT_OK;
  }

  void fill_camera(size_t s) {
    const SceneRes& r = *scenes[s];
    CameraParams& cp = h_cams.p[s];
    matmul_f32(r.proj, r.view, cp.PV);
    cp.cam_pos[0] = r.view[12];  // glm::column(view, 3), renderer.cpp:279
    cp.cam_pos[1] = r.view[13];
    cp.cam_pos[2] = r.view[14];
    cp.W = r.W;
    cp.H = r.H;
  }

  // The frame's work, stream-ordered (also the body of the captured graph;
  // the stage events are recorded as external event nodes there, so that
  // replays still time the stages).
  bool capturing = false;

  cudaError_t record(int k) {
    return capturing ? cudaEventRecordWithFlags(ev[k], stream, cudaEventRecordExternal) : cudaEventRecord(ev[k], stream);
  }

  vct_status encode() {
    const BatchBuffers bb = buffers();
    launches = 0;
    VCT_CUDA(cudaMemcpyAsync(d_cams.p, h_cams.p, scenes.size() * sizeof(CameraParams), cudaMemcpyHostToDevice,
                             stream));
    VCT_CUDA(cudaMemsetAsync(d_status.p, 0, sizeof(FrameStatus), stream));
    VCT_CUDA(record(0));
    BatchWork wb = work(bricks);
    wb.queue = queue.p + 1;  // the brick queue (queue[0] schedules the trace)
    VCT_CUDA(launch_voxelize_batch(work(tris), wb, bricks.total(), cfg.vox_mode, VCT_STORAGE_RGBA8, bb,
                                   scan_tmp.p, shape, sms, stream, &launches));
    VCT_CUDA(record(1));
    if (fused) {
      BatchWork none = work(regions);
      none.total = 0;
      const BatchWork tail[3] = {work(tail4), work(tail5), work(tail6)};
      VCT_CUDA(launch_mipmap_batch(none, tail, 3, 4, VCT_STORAGE_RGBA8, stream, &launches));
    } else {
      const BatchWork tail[2] = {work(tail5), work(tail6)};
      VCT_CUDA(launch_mipmap_batch(work(regions), tail, 2, 5, VCT_STORAGE_RGBA8, stream, &launches));
    }
    VCT_CUDA(launch_occupancy_batch(work(occw), stream, &launches));
    VCT_CUDA(record(2));
    VCT_CUDA(launch_gbuffer_batch(work(tris), work(tiles), total_px, bb, sms, stream, &launches));
    VCT_CUDA(record(3));
    if (shape.trace_per_scene) {
      // Fork the side streams off the frame's stream, trace the scenes
      // round-robin on them (largest first), join back.
      VCT_CUDA(cudaEventRecord(fork_ev, stream));
      for (int k = 0; k < kSide; ++k) VCT_CUDA(cudaStreamWaitEvent(side[k], fork_ev, 0));
      for (size_t i = 0; i < trace_order.size(); ++i) {
        const int s = trace_order[i];
        const SceneRes& r = *scenes[s];
        TraceParams tp = r.tp;
        tp.tile_rows = shape.trace_tile_rows;
        VCT_CUDA(launch_trace(r.sp, h_cams.p[s], r.maps.ms, tp, gb_pos.p + px_base[s], gb_nrm.p + px_base[s],
                              frame.p + px_base[s], nullptr, side[i % kSide], &launches));
      }
      for (int k = 0; k < kSide; ++k) {
        VCT_CUDA(cudaEventRecord(join_ev[k], side[k]));
        VCT_CUDA(cudaStreamWaitEvent(stream, join_ev[k], 0));
      }
    } else {
      VCT_CUDA(launch_trace_batch(work(tiles, true), bb, shape, sms, stream, &launches, cfg.far_share != 0));
    }
    VCT_CUDA(record(4));
    VCT_CUDA(cudaMemcpyAsync(h_status.p, d_status.p, sizeof(FrameStatus), cudaMemcpyDeviceToHost, stream));
    return VCT_OK;
  }

  vct_status submit() {
    if (cfg.use_graph) {
      if (!graph) {
        cudaGraph_t g = nullptr;
        VCT_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        capturing = true;
        const vct_status s = encode();
        capturing = false;
        const cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (s != VCT_OK) {
          if (g) cudaGraphDestroy(g);
          return s;
        }
        VCT_CUDA(e);
        const cudaError_t ie = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        VCT_CUDA(ie);
      }
      VCT_CUDA(cudaGraphLaunch(graph, stream));
    } else {
      VCT_CHECK(encode());
    }
    pending = true;
    have_frame = true;
    return VCT_OK;
  }

  // Wait for the frame; on a work-list overflow grow the list and render
  // the frame again (results are exact once this returns).
  vct_status finish() {
    if (!pending) return VCT_OK;
    for (int attempt = 0; attempt < 4; ++attempt) {
      VCT_CUDA(cudaStreamSynchronize(stream));
      pending = false;
      const FrameStatus s = *h_status.p;
      VCT_CHECK(heavy.grow(s, brick_count.n, stream));  // exact either way: no redo
      bool redo = false;
      if (s.pair_total > pair_list.n) {
        VCT_CHECK(pair_list.ensure((size_t)s.pair_total + s.pair_total / 4 + 4096));
        redo = true;
      }
      if (s.bigtri_total > bin_big_cap) {
        VCT_CHECK(grow_bin_big(s.bigtri_total + s.bigtri_total / 4 + 256));
        redo = true;
      }
      if (s.big_total > rbig_cap) {
        VCT_CHECK(grow_rbig(s.big_total + s.big_total / 4 + 1024));
        redo = true;
      }
      if (!redo) return VCT_OK;
      drop_graph();
      VCT_CHECK(submit());
    }
    return set_error(VCT_ERR_CUDA, "batch work lists kept overflowing");
  }
};

namespace {

vct_status check_scene(const vct_batch_scene& d, uint32_t i) {
  if (d.width < 1 || d.height < 1 || d.width > 16384 || d.height > 16384)
    return set_error(VCT_ERR_INVALID_VALUE, "scene %u: frame %dx%d", i, d.width, d.height);
  if (!is_pow2((uint32_t)d.grid_res) || d.grid_res < 16 || d.grid_res > 256)
    return set_error(VCT_ERR_INVALID_VALUE, "scene %u: grid_res %d (need a power of two in [16, 256])", i,
                     d.grid_res);
  if (d.cone_set != VCT_CONES_REF9 && d.cone_set != VCT_CONES_SIX60)
    return set_error(VCT_ERR_INVALID_VALUE, "scene %u: cone_set %d", i, d.cone_set);
  if (!(d.cube_size > 0.0f)) return set_error(VCT_ERR_INVALID_VALUE, "scene %u: cube_size", i);
  if (!d.materials || d.n_materials < 1) return set_error(VCT_ERR_INVALID_VALUE, "scene %u: no materials", i);
  if (d.n_lights > (uint32_t)kMaxLights || (d.n_lights && !d.lights))
    return set_error(VCT_ERR_INVALID_VALUE, "scene %u: %u lights (at most %d)", i, d.n_lights, kMaxLights);
  if (d.n_meshes && !d.meshes) return set_error(VCT_ERR_INVALID_VALUE, "scene %u: meshes is NULL", i);
  uint64_t tris = 0;
  for (uint32_t m = 0; m < d.n_meshes; ++m) {
    const vct_batch_mesh& ms = d.meshes[m];
    if (ms.n_tris && (!ms.verts || !ms.indices || !ms.tri_material))
      return set_error(VCT_ERR_INVALID_VALUE, "scene %u mesh %u: NULL array", i, m);
    for (uint64_t k = 0; k < 3ull * ms.n_tris; ++k)
      if (ms.indices[k] >= ms.n_verts)
        return set_error(VCT_ERR_INVALID_VALUE, "scene %u mesh %u: index %u >= %u vertices", i, m, ms.indices[k],
                         ms.n_verts);
    for (uint32_t t = 0; t < ms.n_tris; ++t)
      if (ms.tri_material[t] >= d.n_materials)
        return set_error(VCT_ERR_INVALID_ID, "scene %u mesh %u: triangle %u uses material %u of %u", i, m, t,
                         ms.tri_material[t], d.n_materials);
    tris += ms.n_tris;
  }
  if (tris >= (1ull << 31)) return set_error(VCT_ERR_INVALID_VALUE, "scene %u: too many triangles", i);
  return VCT_OK;
}

template <class T>
vct_status upload(DevBuf<T>& d, const T* h, size_t n) {
  VCT_CHECK(d.ensure(std::max<size_t>(n, 1)));
  if (n) VCT_CUDA(cudaMemcpy(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice));
  return VCT_OK;
}

vct_status build_scene(const vct_batch_scene& d, SceneRes& r, int far_share) {
  r.W = d.width;
  r.H = d.height;
  r.N = d.grid_res;
  VCT_CHECK(r.maps.alloc((uint32_t)d.grid_res, VCT_MIP_ANISO, VCT_STORAGE_RGBA8));
  r.L = r.maps.ms.L;
  std::vector<DevInstance> inst(std::max<uint32_t>(d.n_meshes, 1));
  uint32_t base = 0;
  for (uint32_t m = 0; m < d.n_meshes; ++m) {
    const vct_batch_mesh& ms = d.meshes[m];
    r.verts.emplace_back(new DevBuf<vct_vert_data>());
    r.indices.emplace_back(new DevBuf<uint32_t>());
    r.tri_mat.emplace_back(new DevBuf<uint32_t>());
    VCT_CHECK(upload(*r.verts.back(), ms.verts, ms.n_verts));
    VCT_CHECK(upload(*r.indices.back(), ms.indices, 3 * (size_t)ms.n_tris));
    VCT_CHECK(upload(*r.tri_mat.back(), ms.tri_material, ms.n_tris));
    DevInstance& di = inst[m];
    std::memcpy(di.M, ms.model, sizeof(di.M));
    normal_matrix(ms.model, di.NM);
    di.tri_base = base;
    di.n_tris = ms.n_tris;
    di.verts = r.verts.back()->p;
    di.indices = r.indices.back()->p;
    di.tri_obj = r.tri_mat.back()->p;  // the draw object of a triangle is its material
    di.n_verts = ms.n_verts;
    di.pad = 0;
    base += ms.n_tris;
  }
  r.n_tris = base;
  VCT_CHECK(upload(r.inst, inst.data(), inst.size()));
  VCT_CHECK(upload(r.materials, d.materials, d.n_materials));
  std::vector<uint32_t> ident(d.n_materials);
  for (uint32_t k = 0; k < d.n_materials; ++k) ident[k] = k;
  VCT_CHECK(upload(r.identity, ident.data(), ident.size()));
  std::memset(&r.sp, 0, sizeof(r.sp));
  r.sp.inst = r.inst.p;
  r.sp.materials = r.materials.p;
  r.sp.obj_material = r.identity.p;
  r.sp.n_instances = d.n_meshes;
  r.sp.total_tris = base;
  r.sp.n_materials = d.n_materials;
  r.sp.n_lights = (int32_t)d.n_lights;
  r.sp.cube_size = d.cube_size;
  r.sp.radiance_max = 1.0f;
  for (uint32_t l = 0; l < d.n_lights; ++l) r.sp.lights[l] = d.lights[l];
  std::memset(&r.tp, 0, sizeof(r.tp));
  r.tp.enable_direct = r.tp.enable_diffuse = r.tp.enable_specular = r.tp.enable_shadow = 1;
  r.tp.view_voxel_dir = 7;
  r.tp.cone_set = d.cone_set;
  r.tp.sampler = VCT_SAMPLER_HW;
  r.tp.mip_mode = VCT_MIP_ANISO;
  r.tp.far_share = far_share;
  std::memcpy(r.view, d.view, sizeof(r.view));
  std::memcpy(r.proj, d.proj, sizeof(r.proj));
  return VCT_OK;
}

vct_status make_prefix(Prefix& p, const std::vector<uint32_t>& counts) {
  p.h.assign(counts.size() + 1, 0);
  for (size_t i = 0; i < counts.size(); ++i) {
    const uint64_t v = (uint64_t)p.h[i] + counts[i];
    if (v >= 0xffffffffull) return set_error(VCT_ERR_INVALID_VALUE, "batch too large");
    p.h[i + 1] = (uint32_t)v;
  }
  return upload(p.d, p.h.data(), p.h.size());
}

vct_status build_batch(vct_batch* b, const vct_batch_scene* descs, uint32_t n) {
  b->sms = device_sms();
  VCT_CUDA(cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking));
  b->stream = b->own_stream;
  for (auto& e : b->ev) VCT_CUDA(cudaEventCreate(&e));
  VCT_CUDA(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
  for (int k = 0; k < vct_batch::kSide; ++k) {
    VCT_CUDA(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
    VCT_CUDA(cudaEventCreateWithFlags(&b->join_ev[k], cudaEventDisableTiming));
  }
  std::vector<uint32_t> c_tris, c_bricks, c_regions, c_tail4, c_tail5, c_tail6, c_tiles, c_occw;
  uint64_t total_tris = 0;
  for (uint32_t i = 0; i < n; ++i) {
    b->scenes.emplace_back(new SceneRes());
    VCT_CHECK(build_scene(descs[i], *b->scenes.back(), b->cfg.far_share));
    const SceneRes& r = *b->scenes.back();
    const uint32_t nb = (uint32_t)(r.N / kBrick);
    c_tris.push_back((r.n_tris + 31u) & ~31u);
    c_bricks.push_back(nb * nb * nb);
    const uint32_t rg = (uint32_t)(r.N / 16);
    c_regions.push_back(rg * rg * rg);
    const uint32_t s4 = r.L > 4 ? (uint32_t)(r.N >> 4) : 0u;
    const uint32_t s5 = r.L > 5 ? (uint32_t)(r.N >> 5) : 0u, s6 = r.L > 6 ? (uint32_t)(r.N >> 6) : 0u;
    c_tail4.push_back(s4 * s4 * s4);
    c_tail5.push_back(s5 * s5 * s5);  // texels; a thread computes all six maps
    c_tail6.push_back(s6 * s6 * s6);
    c_tiles.push_back((uint32_t)((r.W + 15) / 16) * (uint32_t)((r.H + 15) / 16));
    c_occw.push_back(occupancy_words(r.maps.ms));
    total_tris += r.n_tris;
  }
  VCT_CHECK(make_prefix(b->tris, c_tris));
  VCT_CHECK(make_prefix(b->bricks, c_bricks));
  VCT_CHECK(make_prefix(b->regions, c_regions));
  VCT_CHECK(make_prefix(b->tail4, c_tail4));
  VCT_CHECK(make_prefix(b->tail5, c_tail5));
  VCT_CHECK(make_prefix(b->tail6, c_tail6));
  VCT_CHECK(make_prefix(b->occw, c_occw));
  VCT_CHECK(make_prefix(b->tiles, c_tiles));
  // fused mip levels 1-3 (every scene: RGBA8 anisotropic maps of >= 4 levels)
  b->fused = kFuseBrickMips;
  for (uint32_t i = 0; i < n && b->fused; ++i) b->fused = b->scenes[i]->maps.ms.L >= 4;
  if (b->fused) {
    std::vector<BrickMips> hm(n);
    for (uint32_t i = 0; i < n; ++i) {
      const MapSet& ms = b->scenes[i]->maps.ms;
      BrickMips& bm = hm[i];
      std::memset(&bm, 0, sizeof(bm));
      for (int d = 0; d < 6; ++d)
        for (int l = 1; l <= 3; ++l) bm.surf[d][l] = ms.surf[d][l];
      bm.has_alpha = ms.alpha_tex[0] != 0;
      for (int k = 0; k < 2 && bm.has_alpha; ++k)
        for (int l = 1; l <= 3; ++l) bm.alpha[k][l] = ms.alpha_surf[k][l];
      for (int l = 1; l <= 3 && ms.skip_empty; ++l) bm.occ_raw[l] = ms.occ_raw[l];
    }
    VCT_CHECK(upload(b->d_mips, hm.data(), hm.size()));
  }
  // scene descriptors
  std::vector<BatchScene> hs(n);
  size_t px = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const SceneRes& r = *b->scenes[i];
    BatchScene& s = hs[i];
    std::memset(&s, 0, sizeof(s));
    s.sp = r.sp;
    s.ms = r.maps.ms;
    if (b->fused) {  // occupancy bytes of levels 1-3 from the brick kernel; coarser ones ORed from level 3's
      s.ms.occ_k = 3;
      s.ms.occ_l1_packed = 0;
    }
    s.tp = r.tp;
    s.N = r.N;
    s.W = r.W;
    s.H = r.H;
    s.brick_base = b->bricks.h[i];
    s.px_base = px;
    b->px_base.push_back(px);
    px += (size_t)r.W * r.H;
  }
  b->total_px = px;
  for (uint32_t i = 0; i < n; ++i) b->trace_order.push_back((int)i);
  std::stable_sort(b->trace_order.begin(), b->trace_order.end(), [&](int a, int c) {
    return (size_t)b->scenes[a]->W * b->scenes[a]->H > (size_t)b->scenes[c]->W * b->scenes[c]->H;
  });
  VCT_CHECK(upload(b->d_scenes, hs.data(), hs.size()));
  VCT_CHECK(b->h_cams.ensure(n));
  VCT_CHECK(b->d_cams.ensure(n));
  for (uint32_t i = 0; i < n; ++i) b->fill_camera(i);
  // work arrays
  const size_t nbk = b->bricks.total();
  VCT_CHECK(b->brick_count.ensure(nbk));
  VCT_CHECK(b->brick_offset.ensure(nbk + 1));
  VCT_CHECK(b->brick_cursor.ensure(nbk));
  VCT_CHECK(b->brick_dirty.ensure(nbk));
  VCT_CUDA(cudaMemsetAsync(b->brick_dirty.p, 1, nbk, b->stream));  // the new maps: every brick writes once
  VCT_CHECK(b->heavy.reserve(nbk, 1024, 65536, b->stream));
  VCT_CHECK(b->scan_tmp.ensure(scan_tmp_words(nbk)));
  VCT_CHECK(b->pair_list.ensure((size_t)std::min<uint64_t>(0xffffff00ull, 4ull * total_tris + 65536ull)));
  VCT_CHECK(b->bin_rec.ensure(std::max<size_t>(b->tris.total(), 1)));
  VCT_CHECK(b->bin_big_count.ensure(1));
  VCT_CHECK(b->grow_bin_big(1 << 12));
  VCT_CHECK(b->rbig_count.ensure(2));
  VCT_CHECK(b->grow_rbig(1 << 16));
  VCT_CHECK(b->queue.ensure(2));
  VCT_CHECK(b->vis.ensure(px));
  VCT_CHECK(b->gb_pos.ensure(px));
  VCT_CHECK(b->gb_nrm.ensure(px));
  VCT_CHECK(b->frame.ensure(px));
  VCT_CHECK(b->d_status.ensure(1));
  VCT_CHECK(b->h_status.ensure(1));
  std::memset(b->h_status.p, 0, sizeof(FrameStatus));
  VCT_CUDA(cudaStreamSynchronize(b->stream));  // (the set-up memsets, before the caller may change streams)
  return VCT_OK;
}

}  // namespace

extern "C" vct_status vct_batch_create(const vct_batch_scene* scenes, uint32_t n_scenes, const vct_batch_config* cfg,
                                       vct_batch** out) {
  clear_error();
  if (!out) return set_error(VCT_ERR_INVALID_VALUE, "out is NULL");
  *out = nullptr;
  if (!scenes || n_scenes == 0) return set_error(VCT_ERR_INVALID_VALUE, "no scenes");
  vct_batch_config c;
  std::memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if (c.vox_mode != VCT_VOX_REF_RASTER2X && c.vox_mode != VCT_VOX_CONSERVATIVE)
    return set_error(VCT_ERR_INVALID_VALUE, "vox_mode %d", c.vox_mode);
  if (c.far_share != 0 && c.far_share != 1) return set_error(VCT_ERR_INVALID_VALUE, "far_share %d", c.far_share);
  for (uint32_t i = 0; i < n_scenes; ++i) VCT_CHECK(check_scene(scenes[i], i));
  VCT_CHECK(ensure_device());
  std::unique_ptr<vct_batch> b(new vct_batch());
  b->cfg = c;
  VCT_CHECK(build_batch(b.get(), scenes, n_scenes));
  *out = b.release();
  return VCT_OK;
}

extern "C" void vct_batch_destroy(vct_batch* b) { delete b; }

extern "C" void vct_batch_config_default(vct_batch_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->vox_mode = VCT_VOX_REF_RASTER2X;
  cfg->far_share = 1;
}

extern "C" vct_status vct_batch_set_camera(vct_batch* b, uint32_t scene, const float view[16],
                                           const float proj[16]) {
  clear_error();
  if (!b || !view || !proj) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (scene >= b->scenes.size()) return set_error(VCT_ERR_INVALID_ID, "scene %u of %zu", scene, b->scenes.size());
  VCT_CHECK(b->finish());  // the previous frame has read the camera staging buffer
  std::memcpy(b->scenes[scene]->view, view, 16 * sizeof(float));
  std::memcpy(b->scenes[scene]->proj, proj, 16 * sizeof(float));
  b->fill_camera(scene);
  // The per-scene trace launches take the camera as a kernel parameter,
  // which a captured graph holds by value: capture it again.
  if (b->shape.trace_per_scene) b->drop_graph();
  return VCT_OK;
}

extern "C" vct_status vct_batch_render(vct_batch* b) {
  clear_error();
  if (!b) return set_error(VCT_ERR_INVALID_VALUE, "NULL batch");
  VCT_CHECK(b->finish());
  return b->submit();
}

extern "C" vct_status vct_batch_synchronize(vct_batch* b) {
  clear_error();
  if (!b) return set_error(VCT_ERR_INVALID_VALUE, "NULL batch");
  return b->finish();
}

extern "C" vct_status vct_batch_set_stream(vct_batch* b, void* stream) {
  clear_error();
  if (!b) return set_error(VCT_ERR_INVALID_VALUE, "NULL batch");
  VCT_CHECK(b->finish());
  b->stream = stream ? (cudaStream_t)stream : b->own_stream;
  return VCT_OK;
}

extern "C" vct_status vct_batch_read_frame(vct_batch* b, uint32_t scene, void* rgba8) {
  clear_error();
  if (!b || !rgba8) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (scene >= b->scenes.size()) return set_error(VCT_ERR_INVALID_ID, "scene %u of %zu", scene, b->scenes.size());
  VCT_CHECK(b->finish());
  const SceneRes& r = *b->scenes[scene];
  if (!b->have_frame) {
    std::memset(rgba8, 0, (size_t)r.W * r.H * 4);
    return VCT_OK;
  }
  VCT_CUDA(cudaMemcpyAsync(rgba8, b->frame.p + b->px_base[scene], (size_t)r.W * r.H * sizeof(uchar4),
                           cudaMemcpyDeviceToHost, b->stream));
  VCT_CUDA(cudaStreamSynchronize(b->stream));
  return VCT_OK;
}

extern "C" vct_status vct_batch_read_voxels(vct_batch* b, uint32_t scene, int32_t level, int32_t map, void* rgba8) {
  clear_error();
  if (!b || !rgba8) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (scene >= b->scenes.size()) return set_error(VCT_ERR_INVALID_ID, "scene %u of %zu", scene, b->scenes.size());
  const SceneRes& r = *b->scenes[scene];
  if (level < 0 || level >= r.L) return set_error(VCT_ERR_INVALID_VALUE, "level %d of %d", level, r.L);
  if (map < 0 || map >= 6) return set_error(VCT_ERR_INVALID_VALUE, "map %d", map);
  VCT_CHECK(b->finish());
  cudaArray_t a = r.maps.l0_arr;
  if (level > 0) VCT_CUDA(cudaGetMipmappedArrayLevel(&a, r.maps.dir_arr[map], level - 1));
  const size_t s = (size_t)(r.N >> level);
  cudaMemcpy3DParms p;
  std::memset(&p, 0, sizeof(p));
  p.srcArray = a;
  p.dstPtr = make_cudaPitchedPtr(rgba8, s * 4, s, s);
  p.extent = make_cudaExtent(s, s, s);
  p.kind = cudaMemcpyDeviceToHost;
  VCT_CUDA(cudaMemcpy3DAsync(&p, b->stream));
  VCT_CUDA(cudaStreamSynchronize(b->stream));
  return VCT_OK;
}

extern "C" vct_status vct_batch_stage_times(vct_batch* b, vct_stage_times* out) {
  clear_error();
  if (!b || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  VCT_CHECK(b->finish());
  std::memset(out, 0, sizeof(*out));
  if (!b->have_frame) return VCT_OK;
  float t[4];
  for (int k = 0; k < 4; ++k) VCT_CUDA(cudaEventElapsedTime(&t[k], b->ev[k], b->ev[k + 1]));
  out->voxelize = t[0];
  out->mipmap = t[1];
  out->gbuffer = t[2];
  out->trace = t[3];
  VCT_CUDA(cudaEventElapsedTime(&out->total, b->ev[0], b->ev[4]));
  out->kernel_launches = (uint32_t)b->launches;
  out->voxelized = 1u;
  out->split_bricks = b->h_status.p->heavy_total;
  return VCT_OK;
}

extern "C" vct_status vct_batch_get_shape(vct_batch* b, vct_batch_shape* out) {
  clear_error();
  if (!b || !out) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  out->bin_ctas_per_sm = b->shape.bin_ctas_per_sm;
  out->bricks_ctas_per_sm = b->shape.bricks_ctas_per_sm;
  out->trace_ctas_per_sm = b->shape.trace_ctas_per_sm;
  out->trace_dynamic = b->shape.trace_dynamic;
  out->trace_per_scene = b->shape.trace_per_scene;
  out->trace_tile_rows = b->shape.trace_tile_rows;
  return VCT_OK;
}

extern "C" vct_status vct_batch_set_shape(vct_batch* b, const vct_batch_shape* s) {
  clear_error();
  if (!b || !s) return set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
  if (s->bin_ctas_per_sm < 1 || s->bin_ctas_per_sm > 32 || s->bricks_ctas_per_sm < 1 ||
      s->bricks_ctas_per_sm > 32 || s->trace_ctas_per_sm < 0 || s->trace_ctas_per_sm > 3 ||
      (s->trace_dynamic != 0 && s->trace_dynamic != 1) || (s->trace_per_scene != 0 && s->trace_per_scene != 1) ||
      (s->trace_tile_rows != 8 && s->trace_tile_rows != 16 && s->trace_tile_rows != 32))
    return set_error(VCT_ERR_INVALID_VALUE, "launch shape out of range");
  VCT_CHECK(b->finish());
  b->shape.bin_ctas_per_sm = s->bin_ctas_per_sm;
  b->shape.bricks_ctas_per_sm = s->bricks_ctas_per_sm;
  b->shape.trace_ctas_per_sm = s->trace_ctas_per_sm;
  b->shape.trace_dynamic = s->trace_dynamic;
  b->shape.trace_per_scene = s->trace_per_scene;
  b->shape.trace_tile_rows = s->trace_tile_rows;
  b->drop_graph();  // launch shapes are baked into a captured graph
  return VCT_OK;
}

namespace {

// Mean device time of `frames` frames of the current shape (the first
// frame of a shape is a warm-up: it may capture a graph or grow lists).
vct_status time_frames(vct_batch* b, int frames, float* ms) {
  VCT_CHECK(b->submit());
  VCT_CHECK(b->finish());
  float sum = 0.0f;
  for (int f = 0; f < frames; ++f) {
    VCT_CHECK(b->submit());
    VCT_CHECK(b->finish());
    float t = 0.0f;
    VCT_CUDA(cudaEventElapsedTime(&t, b->ev[0], b->ev[4]));
    sum += t;
  }
  *ms = sum / (float)frames;
  return VCT_OK;
}

}  // namespace

extern "C" vct_status vct_batch_autotune(vct_batch* b, int32_t frames, vct_batch_shape* best, float* ms_before,
                                         float* ms_after) {
  clear_error();
  if (!b) return set_error(VCT_ERR_INVALID_VALUE, "NULL batch");
  if (frames < 1) frames = 3;
  VCT_CHECK(b->finish());
  float base = 0.0f;
  VCT_CHECK(time_frames(b, frames, &base));
  BatchShape cur = b->shape;
  float cur_ms = base;
  // Coordinate search: each field in turn over its candidates, keeping the
  // others at their best values so far.
  const int bin_c[] = {2, 4, 8};
  const int brick_c[] = {2, 4, 8};
  const int trace_c[] = {2, 3};
  const int dyn_c[] = {0, 1};
  auto try_shape = [&](const BatchShape& s) -> vct_status {
    if (std::memcmp(&s, &cur, sizeof(s)) == 0) return VCT_OK;
    b->shape = s;
    b->drop_graph();
    float ms = 0.0f;
    VCT_CHECK(time_frames(b, frames, &ms));
    if (ms < cur_ms) {
      cur_ms = ms;
      cur = s;
    }
    return VCT_OK;
  };
  auto try_field = [&](int BatchShape::*field, const auto& cand) -> vct_status {
    const int nc = (int)(sizeof(cand) / sizeof(cand[0]));
    for (int k = 0; k < nc; ++k) {
      BatchShape s = cur;
      s.*field = cand[k];
      VCT_CHECK(try_shape(s));
    }
    return VCT_OK;
  };
  // The trace's form first, from the same starting point: one launch per
  // scene (16x8 or, with shared far fields, 16x16 or 16x32 tiles), one
  // launch with one CTA per tile, or one persistent launch (2 or 3 CTAs
  // per SM).
  {
    const BatchShape start = cur;
    BatchShape forms[6];
    int nf = 0;
    for (int rows = 8; rows <= 32; rows *= 2) {
      if (rows > 8 && !b->cfg.far_share) continue;
      forms[nf] = start;
      forms[nf].trace_per_scene = 1;
      forms[nf++].trace_tile_rows = rows;
    }
    for (int c : {0, 2, 3}) {
      forms[nf] = start;
      forms[nf].trace_per_scene = 0;
      forms[nf++].trace_ctas_per_sm = c;
    }
    for (int k = 0; k < nf; ++k) VCT_CHECK(try_shape(forms[k]));
  }
  if (!cur.trace_per_scene && cur.trace_ctas_per_sm) {  // the persistent form's scheduling
    VCT_CHECK(try_field(&BatchShape::trace_dynamic, dyn_c));
    VCT_CHECK(try_field(&BatchShape::trace_ctas_per_sm, trace_c));
  }
  VCT_CHECK(try_field(&BatchShape::bricks_ctas_per_sm, brick_c));
  VCT_CHECK(try_field(&BatchShape::bin_ctas_per_sm, bin_c));
  b->shape = cur;
  b->drop_graph();
  if (best) {
    best->bin_ctas_per_sm = cur.bin_ctas_per_sm;
    best->bricks_ctas_per_sm = cur.bricks_ctas_per_sm;
    best->trace_ctas_per_sm = cur.trace_ctas_per_sm;
    best->trace_dynamic = cur.trace_dynamic;
    best->trace_per_scene = cur.trace_per_scene;
    best->trace_tile_rows = cur.trace_tile_rows;
  }
  if (ms_before) *ms_before = base;
  if (ms_after) *ms_after = cur_ms;
  return VCT_OK;
}
