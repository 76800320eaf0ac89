// Batched imaging of masks of uneven sizes, captured in one CUDA graph, with a
// per-size-class autotuner.
//
// Items are grouped by size class (a kernel set and its period L) and, inside a
// class, into sub-batches of equal mask size.  Each sub-batch runs the window
// DFT on its own masks (a mask smaller than the period is centred in it, the
// createMask convention of common/mask.cpp:31-60: the window DFT only needs the
// mask's own pixels and its offset in the period); the SOCS and interpolation
// stages then run once per class over all its images.  Window partials of a
// class share one array with a common parts stride (unused parts are zeroed at
// the start of every run).
//
// Autotuning (LITHO_BATCH_AUTOTUNE) times, per class, every candidate of
//   conv grid N in {nextPow2(4N+1), 2x that} (the FFT plan of the SOCS stage),
//   kernels per CTA in {2, 3, 4, 6, 8, 12} (the SOCS tile), and
//   window column splits in {1, 2}
// with CUDA events on the context's stream and keeps the fastest; results are
// cached on the context by (L, Nx, nk, images, precision).  The plan then
// captures the whole sequence in a CUDA graph (LITHO_BATCH_GRAPH).
#include "litho_internal.cuh"

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

namespace litho {

struct SubBatch {
  int cls, mLx, mLy, count, first_in_class;
  float* masks;
};

struct ClassRun {
  int L = 0;
  const litho_kernel_set* ks = nullptr;
  int count = 0, maxM = 0;
  float* images = nullptr;
  DevBuf win, band, tmbuf, wsum;
  int convN = 0, kpg = 1, colSplits = 1, part_stride = 1;  // convN == 0: the TCC band (band_tcc.cu)
  double tuned_ms = -1.0;
  int candidates = 0;
};

struct TuneKey {
  int L, Nx, nk, count, prec, band;
  bool operator<(const TuneKey& o) const {
    return std::tie(L, Nx, nk, count, prec, band) < std::tie(o.L, o.Nx, o.nk, o.count, o.prec, o.band);
  }
};
struct TuneVal {
  int convN, kpg, colSplits;
  double ms;
};
static std::map<TuneKey, TuneVal> g_tune_cache;  // shared by all contexts of the process

}  // namespace litho

struct litho_batch_plan {
  litho_ctx* ctx = nullptr;
  int precision = LITHO_PREC_FP32, flags = 0;
  std::vector<litho::SubBatch> subs;
  std::vector<litho::ClassRun> classes;
  std::vector<float*> item_mask, item_image;
  litho::DevBuf mask_pool, image_pool;
  // the window DFTs of a class's sub-batches run as parallel branches: streams for all
  // but the largest, a fork event and one join event per branch
  std::vector<cudaStream_t> wstreams;
  std::vector<cudaEvent_t> wevents;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace litho {

static ImgGeom class_geom(const ClassRun& c, int convN) {
  return ImgGeom{c.L, c.L, c.L, c.L, c.ks->Nx, c.ks->Ny, c.ks->nk, convN};
}

static int default_conv(int Nx, int Ny) {
  const int n = next_pow2(4 * std::max(Nx, Ny) + 1);
  return n < 32 ? 32 : n;
}

// Switch the context's launch stream for a scope (the stage timers follow it).
struct StreamScope {
  litho_ctx* ctx;
  cudaStream_t saved;
  StreamScope(litho_ctx* c, cudaStream_t s) : ctx(c), saved(c->stream) { c->stream = s; }
  ~StreamScope() { ctx->stream = saved; }
};

// enqueue one class on the context's stream: windows of its sub-batches, SOCS,
// interpolation
static int run_class(litho_batch_plan* bp, int ci) {
  litho_ctx* ctx = bp->ctx;
  ClassRun& c = bp->classes[ci];
  const bool tc = bp->precision == LITHO_PREC_MIXED;
  const int Nx = c.ks->Nx, Ny = c.ks->Ny, KY = 2 * Ny + 1;
  LITHO_CUDA_TRY(ctx, cudaMemsetAsync(c.win.p, 0, (size_t)c.count * c.part_stride * KY * (Nx + 1) * sizeof(float2),
                                      ctx->stream));
  // The sub-batches' window DFTs (one per mask size; each writes its own images'
  // partials).  Mixed form: one persistent launch over up to WIN_MAX_SIZES mask sizes, so
  // that the small sizes' few tiles share the SMs with the large ones'.  Plain form:
  // parallel branches, the largest on the context's stream: all of them stream masks from
  // HBM, so each fills the others' ramps and tails.
  std::vector<const SubBatch*> sb;
  for (const SubBatch& s : bp->subs)
    if (s.cls == ci) sb.push_back(&s);
  std::stable_sort(sb.begin(), sb.end(), [](const SubBatch* a, const SubBatch* b) {
    return (size_t)a->count * a->mLx * a->mLy > (size_t)b->count * b->mLx * b->mLy;
  });
  auto win_plan = [&](const SubBatch& s) {
    ImgGeom gw{s.mLx, s.mLy, c.L, c.L, Nx, Ny, c.ks->nk, c.convN};
    ImgPlan pw = make_plan(gw, s.count, ctx->sm_count);
    pw.colSplits = std::min(c.colSplits, std::max(1, tc ? (s.mLx + 63) / 64 / 2 : (s.mLx + 63) / 64));
    pw.part_stride = c.part_stride;
    return pw;
  };
  if (tc) {
    std::vector<WinPart> parts;
    for (const SubBatch* s : sb) parts.push_back(WinPart{win_plan(*s), s->masks, s->first_in_class});
    for (size_t i = 0; i < parts.size(); i += WIN_MAX_SIZES)
      LITHO_RET(run_win_dft_tc_multi(ctx, parts.data() + i, (int)std::min<size_t>(WIN_MAX_SIZES, parts.size() - i),
                                     c.win.as<float2>()));
  } else {
    if (sb.size() > 1) {
      // tables shared between sub-batches are built here, before the fork
      for (const SubBatch* s : sb) LITHO_RET(prepare_win_dft(ctx, win_plan(*s)));
      LITHO_CUDA_TRY(ctx, cudaEventRecord(bp->wevents[0], ctx->stream));
      for (size_t k = 1; k < sb.size(); ++k)
        LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(bp->wstreams[k - 1], bp->wevents[0], 0));
    }
    for (size_t k = 0; k < sb.size(); ++k) {
      const SubBatch& s = *sb[k];
      StreamScope scope(ctx, k == 0 ? ctx->stream : bp->wstreams[k - 1]);
      float2* wp = c.win.as<float2>() + (size_t)s.first_in_class * c.part_stride * KY * (Nx + 1);
      LITHO_RET(run_win_dft(ctx, win_plan(s), s.masks, wp));
      if (k > 0) LITHO_CUDA_TRY(ctx, cudaEventRecord(bp->wevents[k], ctx->stream));
    }
    for (size_t k = 1; k < sb.size(); ++k) LITHO_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, bp->wevents[k], 0));
  }
  const bool band = c.convN == 0;
  ImgPlan p = make_plan(class_geom(c, band ? default_conv(Nx, Ny) : c.convN), c.count, ctx->sm_count);
  p.kpg = band ? c.ks->nk : std::min(c.kpg, c.ks->nk);
  p.ngroups = band ? c.ks->band_nc : (c.ks->nk + p.kpg - 1) / p.kpg;
  WindowSrc w;
  w.part = c.win.as<float2>();
  w.nparts = c.part_stride;
  if (band) LITHO_RET(run_band_tcc(ctx, p, w, c.ks, c.wsum.as<float2>(), c.band.as<float2>()));
  else LITHO_RET(run_socs(ctx, p, w, c.ks->krn, c.ks->scales, c.band.as<float2>(), nullptr));
  if (tc) return run_fi_tc(ctx, p, c.band.as<float2>(), c.tmbuf.as<float>(), c.images);
  return run_fi(ctx, p, c.band.as<float2>(), c.tmbuf.as<float>(), c.images);
}

// Every class with masks, one after another on the context's stream.  (Running the
// classes as parallel graph branches, plain or staggered so that one class's SOCS meets
// another's streaming kernels, with the persistent kernels taking tiles from per-class
// counters, measured slower: the streaming kernels hold ~200 KB of shared memory per
// SM, so a class's latency-bound SOCS CTAs and another class's streaming CTAs cannot
// share an SM, and whichever kernel was launched first takes the SMs as they free up.)
static int run_all(litho_batch_plan* bp) {
  for (int ci = 0; ci < (int)bp->classes.size(); ++ci)
    if (bp->classes[ci].count > 0) LITHO_RET(run_class(bp, ci));
  return LITHO_OK;
}

static int time_class(litho_batch_plan* bp, int ci, float* ms, int reps = 3) {
  litho_ctx* ctx = bp->ctx;
  cudaEvent_t a, b;
  LITHO_CUDA_TRY(ctx, cudaEventCreate(&a));
  LITHO_CUDA_TRY(ctx, cudaEventCreate(&b));
  int rc = run_class(bp, ci);  // warm (tables, workspaces)
  float best = 1e30f;
  for (int r = 0; r < reps && rc == LITHO_OK; ++r) {
    cudaEventRecord(a, ctx->stream);
    rc = run_class(bp, ci);
    cudaEventRecord(b, ctx->stream);
    if (cudaEventSynchronize(b) != cudaSuccess) rc = LITHO_ERR_CUDA;
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    best = std::min(best, t);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = best;
  return rc;
}

static int tune_class(litho_batch_plan* bp, int ci) {
  ClassRun& c = bp->classes[ci];
  const bool band_ok = band_tcc_available(bp->ctx, c.ks);
  const int method = band_ok ? (bp->ctx->band_method == LITHO_BAND_TCC ? 2 : 1) : 0;
  const TuneKey key{c.L, c.ks->Nx, c.ks->nk, c.count, bp->precision, method};
  auto it = g_tune_cache.find(key);
  if (it != g_tune_cache.end()) {
    c.convN = it->second.convN;
    c.kpg = it->second.kpg;
    c.colSplits = it->second.colSplits;
    c.tuned_ms = it->second.ms;
    return LITHO_OK;
  }
  // band forms: conv grids of the FFT form, and 0 for the TCC band where the kernel set
  // has a table (with LITHO_BAND_TCC the TCC band alone)
  const int n0 = default_conv(c.ks->Nx, c.ks->Ny);
  std::vector<int> convs;
  if (method != 2) {
    convs.push_back(n0);
    if (2 * n0 <= 128) convs.push_back(2 * n0);
  }
  if (band_ok) convs.push_back(0);
  std::vector<int> kpgs;
  for (int k : {2, 3, 4, 6, 8, 12})
    if (k <= c.ks->nk) kpgs.push_back(k);
  if (kpgs.empty()) kpgs.push_back(1);
  std::vector<int> splits{1, 2};
  // the best candidate of each band form (FFT grids, TCC band) ...
  TuneVal best_fft{convs[0], kpgs[0], 1, 1e30}, best_tcc{0, kpgs[0], 1, 1e30};
  for (int cn : convs)
    for (int k : kpgs)
      for (int sp : splits) {
        if (cn == 0 && k != kpgs[0]) continue;  // kernels per CTA do not apply to the TCC band
        c.convN = cn;
        c.kpg = k;
        c.colSplits = sp;
        float ms = 0.f;
        LITHO_RET(time_class(bp, ci, &ms));
        ++c.candidates;
        TuneVal& b = cn == 0 ? best_tcc : best_fft;
        if (ms < b.ms) b = TuneVal{cn, k, sp, ms};
      }
  // ... then the two finalists timed again, alternately and longer, so that the many FFT
  // candidates' best-of-three does not win on timing noise alone
  TuneVal best = best_fft.ms < best_tcc.ms ? best_fft : best_tcc;
  if (best_fft.ms < 1e29 && best_tcc.ms < 1e29) {
    float f = 1e30f, t = 1e30f;
    for (int round = 0; round < 3; ++round)
      for (TuneVal* v : {&best_fft, &best_tcc}) {
        c.convN = v->convN;
        c.kpg = v->kpg;
        c.colSplits = v->colSplits;
        float ms = 0.f;
        LITHO_RET(time_class(bp, ci, &ms, 5));
        (v == &best_fft ? f : t) = std::min(v == &best_fft ? f : t, ms);
      }
    best_fft.ms = f;
    best_tcc.ms = t;
    best = f < t ? best_fft : best_tcc;
  }
  c.convN = best.convN;
  c.kpg = best.kpg;
  c.colSplits = best.colSplits;
  c.tuned_ms = best.ms;
  g_tune_cache[key] = best;
  return LITHO_OK;
}

}  // namespace litho

using namespace litho;

extern "C" {

int litho_batch_plan_create(litho_ctx* ctx, const litho_kernel_set* const* sets, const int* periods, int nsets,
                            const litho_batch_item* items, int n, int precision, int flags,
                            litho_batch_plan** out) {
  if (ctx == nullptr || out == nullptr) return LITHO_ERR_ARG;
  *out = nullptr;
  LITHO_ARG_CHECK(ctx, sets && periods && items && nsets >= 1 && n >= 1, "bad batch description");
  LITHO_ARG_CHECK(ctx, precision == LITHO_PREC_FP32 || precision == LITHO_PREC_MIXED, "bad precision");
  for (int c = 0; c < nsets; ++c) {
    LITHO_ARG_CHECK(ctx, sets[c] && sets[c]->ctx == ctx, "kernel set %d missing or from another context", c);
    LITHO_ARG_CHECK(ctx, is_pow2(periods[c]) && periods[c] >= 32 && periods[c] <= 16384,
                    "period %d must be a power of two in [32, 16384]", periods[c]);
    LITHO_ARG_CHECK(ctx, sets[c]->Nx <= 16 && sets[c]->Ny <= 16, "kernel half-support must be <= 16");
    LITHO_ARG_CHECK(ctx, 2 * sets[c]->Nx + 1 <= periods[c], "kernel support exceeds the period");
  }
  for (int i = 0; i < n; ++i) {
    const litho_batch_item& it = items[i];
    LITHO_ARG_CHECK(ctx, it.cls >= 0 && it.cls < nsets, "item %d: class %d out of range", i, it.cls);
    LITHO_ARG_CHECK(ctx, it.mLx >= 2 && it.mLy >= 2 && it.mLx <= periods[it.cls] && it.mLy <= periods[it.cls],
                    "item %d: mask %dx%d not within its period %d", i, it.mLx, it.mLy, periods[it.cls]);
    LITHO_ARG_CHECK(ctx, ((periods[it.cls] - it.mLx) % 2) == 0 && ((periods[it.cls] - it.mLy) % 2) == 0,
                    "item %d: period - mask size must be even (centred embedding)", i);
    if (precision == LITHO_PREC_MIXED)
      LITHO_ARG_CHECK(ctx, (it.mLx % 4) == 0, "item %d: mixed precision needs mLx %% 4 == 0 (TMA rows)", i);
  }
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  litho_batch_plan* bp = new litho_batch_plan();
  bp->ctx = ctx;
  bp->precision = precision;
  bp->flags = flags;
  bp->classes.resize(nsets);
  for (int c = 0; c < nsets; ++c) {
    bp->classes[c].L = periods[c];
    bp->classes[c].ks = sets[c];
    bp->classes[c].convN = default_conv(sets[c]->Nx, sets[c]->Ny);
    bp->classes[c].kpg = std::max(1, std::min(4, sets[c]->nk));
  }
  // sub-batches: (class, mLy, mLx) groups in first-appearance order
  std::vector<int> sub_of(n);
  for (int i = 0; i < n; ++i) {
    int s = -1;
    for (int k = 0; k < (int)bp->subs.size(); ++k)
      if (bp->subs[k].cls == items[i].cls && bp->subs[k].mLx == items[i].mLx && bp->subs[k].mLy == items[i].mLy) {
        s = k;
        break;
      }
    if (s < 0) {
      bp->subs.push_back(SubBatch{items[i].cls, items[i].mLx, items[i].mLy, 0, 0, nullptr});
      s = (int)bp->subs.size() - 1;
    }
    sub_of[i] = s;
    bp->subs[s].count++;
  }
  // slots: masks per sub-batch, images per class in sub-batch order
  size_t mask_floats = 0, image_floats = 0;
  for (auto& s : bp->subs) mask_floats += (size_t)s.count * s.mLx * s.mLy;
  for (auto& s : bp->subs) {
    ClassRun& c = bp->classes[s.cls];
    s.first_in_class = c.count;
    c.count += s.count;
    c.maxM = std::max(c.maxM, s.mLy);
  }
  for (auto& c : bp->classes) image_floats += (size_t)c.count * c.L * c.L;
  int rc = bp->mask_pool.ensure(ctx, mask_floats * sizeof(float));
  if (rc == LITHO_OK) rc = bp->image_pool.ensure(ctx, image_floats * sizeof(float));
  if (rc != LITHO_OK) {
    litho_batch_plan_destroy(bp);
    return rc;
  }
  {
    float* mp = bp->mask_pool.as<float>();
    for (auto& s : bp->subs) {
      s.masks = mp;
      mp += (size_t)s.count * s.mLx * s.mLy;
    }
    float* ip = bp->image_pool.as<float>();
    for (auto& c : bp->classes) {
      c.images = ip;
      ip += (size_t)c.count * c.L * c.L;
    }
  }
  bp->item_mask.resize(n);
  bp->item_image.resize(n);
  {
    std::vector<int> used(bp->subs.size(), 0);
    for (int i = 0; i < n; ++i) {
      SubBatch& s = bp->subs[sub_of[i]];
      const int k = used[sub_of[i]]++;
      bp->item_mask[i] = s.masks + (size_t)k * s.mLx * s.mLy;
      ClassRun& c = bp->classes[s.cls];
      bp->item_image[i] = c.images + (size_t)(s.first_in_class + k) * c.L * c.L;
    }
  }
  // per-class workspaces sized for every tuning candidate
  for (auto& c : bp->classes) {
    if (c.count == 0) continue;
    const int Nx = c.ks->Nx, Ny = c.ks->Ny, KY = 2 * Ny + 1;
    c.part_stride = ((c.maxM + 127) / 128) * 2;  // row blocks x up to two column splits
    rc = c.win.ensure(ctx, (size_t)c.count * c.part_stride * KY * (Nx + 1) * sizeof(float2));
    const int groups = std::max(c.ks->nk, c.ks->band_nc);  // the FFT form's kernel groups or the band chunks
    if (rc == LITHO_OK) rc = c.band.ensure(ctx, (size_t)c.count * groups * KY * (4 * Nx + 1) * sizeof(float2));
    const ImgGeom g = class_geom(c, c.convN);
    if (rc == LITHO_OK && c.ks->band_nc > 0) rc = c.wsum.ensure(ctx, band_wsum_bytes(g, c.count));
    const size_t tmb = precision == LITHO_PREC_MIXED ? fi_tc_workspace_bytes(g, c.count)
                                                     : (size_t)c.count * (4 * Ny + 1) * c.L * sizeof(float);
    if (rc == LITHO_OK) rc = c.tmbuf.ensure(ctx, tmb);
    if (rc != LITHO_OK) {
      litho_batch_plan_destroy(bp);
      return rc;
    }
  }
  // branch streams and events for the sub-batches' window DFTs (as many as the largest
  // class has sub-batches)
  {
    std::vector<int> per(nsets, 0);
    int most = 0;
    for (const auto& sbt : bp->subs) most = std::max(most, ++per[sbt.cls]);
    for (int k = 0; k < most && rc == LITHO_OK; ++k) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = LITHO_ERR_CUDA;
      else bp->wevents.push_back(e);
      if (rc == LITHO_OK && k > 0) {
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) rc = LITHO_ERR_CUDA;
        else bp->wstreams.push_back(st);
      }
    }
    if (rc != LITHO_OK) {
      litho_batch_plan_destroy(bp);
      return rc;
    }
  }
  // zero the mask slots so tuning runs read defined data
  if (cudaMemsetAsync(bp->mask_pool.p, 0, mask_floats * sizeof(float), ctx->stream) != cudaSuccess) {
    litho_batch_plan_destroy(bp);
    return LITHO_ERR_CUDA;
  }
  const bool saved_timing = ctx->timing;
  ctx->timing = false;
  if (flags & LITHO_BATCH_AUTOTUNE)
    for (int ci = 0; ci < nsets && rc == LITHO_OK; ++ci)
      if (bp->classes[ci].count > 0) rc = tune_class(bp, ci);
  if (rc == LITHO_OK) rc = run_all(bp);  // warm: every table and attribute exists before capture
  if (rc == LITHO_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = LITHO_ERR_CUDA;
  if (rc == LITHO_OK && (flags & LITHO_BATCH_GRAPH)) {
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      rc = LITHO_ERR_CUDA;
    } else {
      const int rr = run_all(bp);
      const cudaError_t e = cudaStreamEndCapture(ctx->stream, &bp->graph);
      if (rr != LITHO_OK || e != cudaSuccess) rc = rr != LITHO_OK ? rr : LITHO_ERR_CUDA;
      else if (cudaGraphInstantiate(&bp->exec, bp->graph, 0) != cudaSuccess) rc = LITHO_ERR_CUDA;
    }
  }
  ctx->timing = saved_timing;
  if (rc != LITHO_OK) {
    if (ctx->last_error.empty()) set_error(ctx, rc, "batch plan set-up failed");
    litho_batch_plan_destroy(bp);
    return rc;
  }
  *out = bp;
  return LITHO_OK;
}

float* litho_batch_plan_mask(litho_batch_plan* bp, int i) {
  return (bp && i >= 0 && i < (int)bp->item_mask.size()) ? bp->item_mask[i] : nullptr;
}

float* litho_batch_plan_image(litho_batch_plan* bp, int i) {
  return (bp && i >= 0 && i < (int)bp->item_image.size()) ? bp->item_image[i] : nullptr;
}

int litho_batch_plan_run(litho_batch_plan* bp) {
  if (bp == nullptr) return LITHO_ERR_ARG;
  litho_ctx* ctx = bp->ctx;
  LITHO_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (bp->exec) {
    // graph launches are counted as the kernels they contain
    for (auto& c : bp->classes)
      if (c.count > 0) {
        for (auto& s : bp->subs)
          if (&bp->classes[s.cls] == &c) ctx->stage_launches[LITHO_STAGE_WIN_DFT] += 1;
        ctx->stage_launches[LITHO_STAGE_SOCS] += 1;
        ctx->stage_launches[LITHO_STAGE_FI_PREP] += 1;
        ctx->stage_launches[LITHO_STAGE_FI_OUT] += 1;
      }
    LITHO_CUDA_TRY(ctx, cudaGraphLaunch(bp->exec, ctx->stream));
    return LITHO_OK;
  }
  return run_all(bp);
}

int litho_batch_plan_describe(const litho_batch_plan* bp, char* buf, int cap) {
  if (bp == nullptr || buf == nullptr || cap <= 0) return -1;
  std::string s = "{\"graph\": ";
  s += bp->exec ? "true" : "false";
  s += ", \"classes\": [";
  bool first = true;
  for (const auto& c : bp->classes) {
    if (c.count == 0) continue;
    char t[512];
    snprintf(t, sizeof t,
             "%s{\"period\": %d, \"Nx\": %d, \"nk\": %d, \"images\": %d, \"band\": \"%s\", \"conv_n\": %d, "
             "\"kernels_per_cta\": %d, \"band_chunks\": %d, \"window_col_splits\": %d, \"tuned_ms\": %.4f, "
             "\"candidates\": %d}",
             first ? "" : ", ", c.L, c.ks->Nx, c.ks->nk, c.count, c.convN == 0 ? "tcc" : "fft", c.convN,
             c.convN == 0 ? 0 : c.kpg, c.convN == 0 ? c.ks->band_nc : 0, c.colSplits, c.tuned_ms, c.candidates);
    s += t;
    first = false;
  }
  s += "], \"sub_batches\": [";
  for (size_t i = 0; i < bp->subs.size(); ++i) {
    char t[128];
    snprintf(t, sizeof t, "%s{\"period\": %d, \"mask\": %d, \"count\": %d}", i ? ", " : "",
             bp->classes[bp->subs[i].cls].L, bp->subs[i].mLx, bp->subs[i].count);
    s += t;
  }
  s += "]}";
  const int n = (int)std::min<size_t>(s.size(), (size_t)cap - 1);
  memcpy(buf, s.data(), n);
  buf[n] = 0;
  return n;
}

int litho_batch_plan_destroy(litho_batch_plan* bp) {
  if (bp == nullptr) return LITHO_ERR_ARG;
  cudaSetDevice(bp->ctx->device);
  cudaStreamSynchronize(bp->ctx->stream);
  if (bp->exec) cudaGraphExecDestroy(bp->exec);
  if (bp->graph) cudaGraphDestroy(bp->graph);
  for (auto& c : bp->classes) {
    c.win.release();
    c.band.release();
    c.tmbuf.release();
    c.wsum.release();
  }
  for (cudaStream_t st : bp->wstreams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (cudaEvent_t e : bp->wevents) cudaEventDestroy(e);
  bp->mask_pool.release();
  bp->image_pool.release();
  delete bp;
  return LITHO_OK;
}

}  // extern "C"
