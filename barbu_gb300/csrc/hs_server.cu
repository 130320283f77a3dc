// hs_server.cu -- served stream: grooms arrive, are admitted into a device
// slab pool by HBM bytes, are advanced together tick by tick, and leave.
//
// Memory. The server reserves its whole budget in one device allocation at
// creation and carves each groom's state block (positions, velocities,
// rest roots) out of it with a first-fit allocator over 256-byte units;
// freed blocks coalesce with their neighbours. Admission never calls
// cudaMalloc, so a tick's latency does not depend on the CUDA runtime's
// allocator.
//
// Ticks. hs_server_tick retires grooms that have done their frames,
// admits queued requests in arrival order while the budget allows, and
// advances every active groom one frame with the batched path
// (hs_batch.cu: one graph launch). A newly admitted groom is set up on a
// separate admission stream while the tick's frame runs, and joins the
// frames from the next tick on: its set-up overlaps the others' work.
// Admission is first come, first served: a request that does not fit
// waits, and so do those behind it.
//
// Inputs. A request carries its initial spheres, its wind swing and its
// roots (pinned, rigid or skinned; a skinned request brings its bone
// influences, kept in the groom's slab block). Between ticks the caller can
// move a groom's spheres, root transform or bone palette by ticket
// (hs_server_set_*): the values reach the groom's next frame, through the
// tick's table copy. A groom's frames depend only on its own inputs and
// its own elapsed time, so they are the same alone and in a mix, bit for
// bit. A skinned groom waits, without advancing, until it has a palette.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <unordered_map>
#include <vector>

#include "hairsim.h"
#include "hs_api_internal.h"
#include "hs_batch.h"
#include "hs_internal.h"

namespace {

using namespace hs;

constexpr size_t kUnit = 256;

// First-fit allocator over [0, capacity) in kUnit units.
class SlabPool {
 public:
  void reset(size_t capacity) {
    free_.clear();
    cap_ = capacity / kUnit * kUnit;
    if (cap_) free_[0] = cap_;
    used_ = 0;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = (bytes + kUnit - 1) / kUnit * kUnit;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rem = it->second - bytes;
        const size_t at = it->first + bytes;
        free_.erase(it);
        if (rem) free_[at] = rem;
        used_ += bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + kUnit - 1) / kUnit * kUnit;
    used_ -= bytes;
    auto next = free_.lower_bound(off);
    if (next != free_.end() && off + bytes == next->first) {
      bytes += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += bytes;
        return;
      }
    }
    free_[off] = bytes;
  }
  size_t used() const { return used_; }
  size_t capacity() const { return cap_; }

 private:
  std::map<size_t, size_t> free_;  // offset -> size
  size_t cap_ = 0, used_ = 0;
};

struct Request {
  uint64_t ticket = 0;
  std::vector<float> roots, normals, lengths, spheres;  // strand rows in the stored order
  std::vector<uint32_t> order, inv;  // stored -> caller strand index (`stride` entries), and back
  std::vector<uint4> skin;          // SKINNED: packed influences, `stride` entries, stored order
  uint32_t skin_max_bone = 0;
  float m[16] = {};                 // RIGID: transform for the next frame
  float dq[8 * HS_MAX_BONES] = {};  // SKINNED: palette for the next frame
  uint32_t nbones = 0;
  bool has_palette = false;
  hs_strand_params strand{};
  hs_sim_params sim{};
  uint32_t nstrands = 0, frames = 0, keep = 0;
  float wind[3] = {0, 0, 0};
  float swing_amp = 0, swing_omega = 0;
  uint32_t state = HS_REQ_QUEUED;
  uint32_t frames_done = 0;
  hs_groom* groom = nullptr;
  size_t slab_off = 0, slab_bytes = 0;
  bool ready = false;  // set-up finished: advanced from the next tick
};

}  // namespace

struct hs_server {
  hs_ctx* ctx = nullptr;
  hs_server_config cfg{};
  char* d_pool = nullptr;
  SlabPool pool;
  cudaStream_t admit_stream = nullptr;
  cudaEvent_t admit_done = nullptr;
  // Set-up staging: roots, normals, lengths (pinned host, device).
  float* h_stage = nullptr;
  float* d_stage = nullptr;
  size_t stage_floats = 0;
  uint64_t next_ticket = 1;
  std::deque<Request*> queue;
  std::vector<Request*> resident;  // admitted, in admission order
  std::unordered_map<uint64_t, Request*> by_ticket;
  std::vector<hs_groom*> active;   // scratch for the tick: the grooms advanced
  std::vector<Request*> advancing; // and their requests
};

namespace {

void release_request(hs_server* S, Request* r) {
  if (r->groom) {
    if (!r->skin.empty()) r->groom->d_skin = nullptr;  // in the slab block, not its own allocation
    S->ctx->grooms.erase(r->groom);
    free_groom(r->groom);
    r->groom = nullptr;
  }
  if (r->slab_bytes) S->pool.release(r->slab_off, r->slab_bytes);
  r->slab_bytes = 0;
}

// Grows the set-up staging to hold `floats` floats.
hs_status ensure_stage(hs_server* S, size_t floats) {
  if (floats <= S->stage_floats) return HS_OK;
  cudaError_t e = cudaStreamSynchronize(S->admit_stream);
  if (e != cudaSuccess) return cuda_fail(e, "server: staging");
  if (S->h_stage) cudaFreeHost(S->h_stage);
  cudaFree(S->d_stage);
  S->h_stage = nullptr;
  S->d_stage = nullptr;
  S->stage_floats = 0;
  size_t cap = 1 << 20;
  while (cap < floats) cap *= 2;
  e = cudaMallocHost(&S->h_stage, sizeof(float) * cap);
  if (e == cudaSuccess) e = cudaMalloc(&S->d_stage, sizeof(float) * cap);
  if (e != cudaSuccess) return cuda_fail(e, "server: staging");
  S->stage_floats = cap;
  return HS_OK;
}

// Admits one request into slab memory and queues its set-up on the
// admission stream. Returns false (and leaves it queued) if it does not fit.
hs_status admit(hs_server* S, Request* r, bool* admitted) {
  *admitted = false;
  const size_t state = groom_state_bytes(r->nstrands, r->strand.points_per_strand);
  const size_t bytes = state + sizeof(uint4) * r->skin.size();
  size_t off = 0;
  if (!S->pool.alloc(bytes, &off)) return HS_OK;
  hs_groom* g = nullptr;
  hs_status st = make_groom_shell(S->ctx, r->nstrands, r->strand.points_per_strand, r->strand.seed, &r->sim, &g);
  if (st != HS_OK) {
    S->pool.release(off, bytes);
    return st;
  }
  place_groom(g, S->d_pool + off, true);
  r->groom = g;
  r->slab_off = off;
  r->slab_bytes = bytes;
  S->ctx->grooms.insert(g);
  st = set_spheres(g, r->spheres.data(), static_cast<uint32_t>(r->spheres.size() / 4));
  if (st != HS_OK) return st;
  std::memcpy(g->m, r->m, sizeof(g->m));
  if (r->has_palette) {
    st = hs_set_bone_dual_quats(g, r->dq, r->nbones);
    if (st != HS_OK) return st;
  }
  g->order = r->order;
  g->inv = r->inv;
  // Stage roots, normals, lengths, influences and the strand order; the
  // previous set-up must be done with the staging before it is overwritten.
  const size_t n3 = 3 * static_cast<size_t>(r->nstrands);
  const size_t nl = (r->lengths.size() + 3) / 4 * 4;  // influences start 16-byte aligned
  const size_t no = 2 * n3 + nl + 4 * r->skin.size();  // order (4-byte words)
  const size_t need = no + r->order.size();
  st = ensure_stage(S, need);
  if (st != HS_OK) return st;
  cudaError_t e = cudaEventSynchronize(S->admit_done);
  if (e != cudaSuccess) return cuda_fail(e, "server: admission");
  std::memcpy(S->h_stage, r->roots.data(), sizeof(float) * n3);
  std::memcpy(S->h_stage + n3, r->normals.data(), sizeof(float) * n3);
  if (!r->lengths.empty()) std::memcpy(S->h_stage + 2 * n3, r->lengths.data(), sizeof(float) * r->lengths.size());
  if (!r->skin.empty()) {
    std::memcpy(S->h_stage + 2 * n3 + nl, r->skin.data(), sizeof(uint4) * r->skin.size());
    g->d_skin = reinterpret_cast<uint4*>(S->d_pool + off + state);
    g->skin_max_bone = r->skin_max_bone;
  }
  std::memcpy(S->h_stage + no, r->order.data(), sizeof(uint32_t) * r->order.size());
  e = cudaMemcpyAsync(S->d_stage, S->h_stage, sizeof(float) * need, cudaMemcpyHostToDevice, S->admit_stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g->d_order, S->d_stage + no, sizeof(uint32_t) * r->order.size(), cudaMemcpyDeviceToDevice,
                        S->admit_stream);
  if (e == cudaSuccess && !r->skin.empty())
    e = cudaMemcpyAsync(g->d_skin, S->d_stage + 2 * n3 + nl, sizeof(uint4) * r->skin.size(),
                        cudaMemcpyDeviceToDevice, S->admit_stream);
  hs_strand_params sp = r->strand;
  sp.lengths = nullptr;
  if (e == cudaSuccess)
    e = init_groom_on_device(g, S->d_stage, S->d_stage + n3, r->lengths.empty() ? nullptr : S->d_stage + 2 * n3, &sp,
                             S->admit_stream);
  if (e == cudaSuccess) e = cudaEventRecord(S->admit_done, S->admit_stream);
  if (e != cudaSuccess) return cuda_fail(e, "server: admission");
  r->state = HS_REQ_RESIDENT;
  r->ready = false;
  *admitted = true;
  return HS_OK;
}

}  // namespace

using namespace hs;

extern "C" {

HS_API hs_status hs_server_create(hs_ctx* ctx, const hs_server_config* cfg, hs_server** out) {
  if (!ctx || !cfg || !out) return fail(HS_ERR_INVALID_ARG, "hs_server_create: null argument");
  HS_ON_DEVICE(ctx, "hs_server_create");
  *out = nullptr;
  if (cfg->budget_bytes < kUnit) return fail(HS_ERR_INVALID_ARG, "hs_server_create: budget too small");
  hs_server* S = new (std::nothrow) hs_server();
  if (!S) return fail(HS_ERR_OUT_OF_MEMORY, "hs_server_create: host allocation");
  S->ctx = ctx;
  S->cfg = *cfg;
  cudaError_t e = cudaMalloc(&S->d_pool, cfg->budget_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->admit_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->admit_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(S->admit_done, S->admit_stream);
  if (e != cudaSuccess) {
    cudaFree(S->d_pool);
    if (S->admit_stream) cudaStreamDestroy(S->admit_stream);
    if (S->admit_done) cudaEventDestroy(S->admit_done);
    delete S;
    cudaGetLastError();
    return cuda_fail(e, "hs_server_create");
  }
  S->pool.reset(cfg->budget_bytes);
  *out = S;
  return HS_OK;
}

HS_API hs_status hs_server_destroy(hs_server* S) {
  if (!S) return fail(HS_ERR_INVALID_ARG, "hs_server_destroy: null server");
  HS_ON_DEVICE(S->ctx, "hs_server_destroy");
  cudaStreamSynchronize(S->admit_stream);
  cudaStreamSynchronize(S->ctx->stream);
  for (auto& kv : S->by_ticket) {
    release_request(S, kv.second);
    delete kv.second;
  }
  S->by_ticket.clear();
  if (S->h_stage) cudaFreeHost(S->h_stage);
  cudaFree(S->d_stage);
  cudaFree(S->d_pool);
  cudaEventDestroy(S->admit_done);
  cudaStreamDestroy(S->admit_stream);
  delete S;
  return HS_OK;
}

HS_API hs_status hs_server_submit(hs_server* S, const hs_request* q, uint64_t* out_ticket) {
  if (!S || !q || !q->root_pos || !q->root_nrm || (q->nspheres && !q->spheres))
    return fail(HS_ERR_INVALID_ARG, "hs_server_submit: null argument");
  HS_ON_DEVICE(S->ctx, "hs_server_submit");
  if (q->nstrands == 0 || q->frames == 0) return fail(HS_ERR_INVALID_ARG, "hs_server_submit: empty request");
  if (q->nspheres > HS_MAX_SPHERES) return fail(HS_ERR_INVALID_ARG, "hs_server_submit: too many spheres");
  if (q->sim.root_mode == HS_ROOT_EXPLICIT)
    return fail(HS_ERR_UNSUPPORTED, "hs_server_submit: served roots are pinned, rigid or skinned");
  if (q->sim.root_mode == HS_ROOT_SKINNED && (!q->skin_bones || !q->skin_weights))
    return fail(HS_ERR_INVALID_ARG, "hs_server_submit: skinned roots need bone influences");
  hs_status st = validate_sim(&q->sim);
  if (st != HS_OK) return st;
  st = validate_strand(&q->strand, q->root_pos, q->root_nrm, q->lengths, q->nstrands);
  if (st != HS_OK) return st;
  const uint32_t N = q->strand.points_per_strand;
  if (N < HS_MIN_POINTS_PER_STRAND || N > HS_MAX_POINTS_PER_STRAND)
    return fail(HS_ERR_INVALID_ARG, "hs_server_submit: points per strand %u", N);
  if (!std::isfinite(q->wind[0]) || !std::isfinite(q->wind[1]) || !std::isfinite(q->wind[2]) ||
      !std::isfinite(q->swing_amp) || !std::isfinite(q->swing_omega))
    return fail(HS_ERR_INVALID_ARG, "hs_server_submit: non-finite wind");
  const uint32_t stride = (q->nstrands + 31u) & ~31u;
  std::vector<uint4> skin;
  uint32_t max_bone = 0;
  if (q->sim.root_mode == HS_ROOT_SKINNED) {
    st = pack_skin(q->skin_bones, q->skin_weights, q->nstrands, stride, &skin, &max_bone, "hs_server_submit");
    if (st != HS_OK) return st;
  }
  const size_t bytes = groom_state_bytes(q->nstrands, N) + sizeof(uint4) * skin.size();
  if (bytes > S->pool.capacity())
    return fail(HS_ERR_ADMISSION_DENIED, "hs_server_submit: %zu bytes exceed the %zu-byte budget", bytes,
                S->pool.capacity());
  Request* r = new (std::nothrow) Request();
  if (!r) return fail(HS_ERR_OUT_OF_MEMORY, "hs_server_submit: host allocation");
  r->ticket = S->next_ticket++;
  // Strand rows are kept in the order the groom will store them in.
  strand_order(q->root_pos, 3, q->nstrands, stride, q->strand.keep_order != 0, &r->order, &r->inv);
  r->roots.resize(3 * static_cast<size_t>(q->nstrands));
  r->normals.resize(3 * static_cast<size_t>(q->nstrands));
  if (q->lengths) r->lengths.resize(q->nstrands);
  for (uint32_t j = 0; j < q->nstrands; ++j) {
    const size_t c = r->order[j];
    for (int a = 0; a < 3; ++a) {
      r->roots[3 * j + a] = q->root_pos[3 * c + a];
      r->normals[3 * j + a] = q->root_nrm[3 * c + a];
    }
    if (q->lengths) r->lengths[j] = q->lengths[c];
  }
  if (!skin.empty()) {
    std::vector<uint4> caller(std::move(skin));
    skin.assign(stride, make_uint4(0u, 0u, 0u, 0u));
    for (uint32_t j = 0; j < q->nstrands; ++j) skin[j] = caller[r->order[j]];
  }
  if (q->nspheres) r->spheres.assign(q->spheres, q->spheres + 4 * static_cast<size_t>(q->nspheres));
  r->strand = q->strand;
  r->strand.lengths = nullptr;
  r->sim = q->sim;
  r->nstrands = q->nstrands;
  r->frames = q->frames;
  r->keep = q->keep_result;
  std::memcpy(r->wind, q->wind, sizeof(r->wind));
  r->swing_amp = q->swing_amp;
  r->swing_omega = q->swing_omega;
  r->skin = std::move(skin);
  r->skin_max_bone = max_bone;
  for (int c = 0; c < 16; ++c) r->m[c] = (c % 5 == 0) ? 1.0f : 0.0f;  // identity until set
  S->queue.push_back(r);
  S->by_ticket[r->ticket] = r;
  if (out_ticket) *out_ticket = r->ticket;
  return HS_OK;
}

HS_API hs_status hs_server_tick(hs_server* S, float dt, hs_tick_stats* out) {
  if (!S) return fail(HS_ERR_INVALID_ARG, "hs_server_tick: null server");
  HS_ON_DEVICE(S->ctx, "hs_server_tick");
  if (!std::isfinite(dt) || !(dt > 0.0f)) return fail(HS_ERR_INVALID_ARG, "hs_server_tick: dt must be > 0");
  const auto t0 = std::chrono::steady_clock::now();
  hs_tick_stats st{};
  // 1. Retire grooms that have done their frames.
  std::vector<Request*> keep;
  keep.reserve(S->resident.size());
  for (Request* r : S->resident) {
    if (r->frames_done >= r->frames && r->state == HS_REQ_RESIDENT) {
      ++st.retired;
      if (r->keep) {
        r->state = HS_REQ_DONE;  // held until collected
      } else {
        release_request(S, r);
        S->by_ticket.erase(r->ticket);
        delete r;
        continue;
      }
    }
    keep.push_back(r);
  }
  S->resident.swap(keep);
  // 2. Grooms whose set-up was queued last tick join the frames now.
  cudaError_t e = cudaSuccess;
  bool pending = false;
  for (Request* r : S->resident) {
    if (r->state == HS_REQ_RESIDENT && !r->ready) {
      r->ready = true;
      pending = true;
    }
  }
  if (pending) e = cudaStreamWaitEvent(S->ctx->stream, S->admit_done, 0);
  if (e != cudaSuccess) return cuda_fail(e, "hs_server_tick: admission wait");
  // 3. Admit queued requests in arrival order while they fit.
  while (!S->queue.empty()) {
    if (S->cfg.max_grooms && S->resident.size() >= S->cfg.max_grooms) break;
    Request* r = S->queue.front();
    bool ok = false;
    hs_status as = admit(S, r, &ok);
    if (as != HS_OK) return as;
    if (!ok) break;
    S->queue.pop_front();
    S->resident.push_back(r);
    ++st.admitted;
  }
  // 4. Advance every active groom one frame (one graph launch).
  S->active.clear();
  S->advancing.clear();
  for (Request* r : S->resident) {
    if (r->state != HS_REQ_RESIDENT || !r->ready) continue;
    if (r->sim.root_mode == HS_ROOT_SKINNED && r->groom->nbones <= r->skin_max_bone) continue;  // no palette yet
    const double t = static_cast<double>(r->frames_done + 1) * dt;
    float w[3] = {r->wind[0] + static_cast<float>(r->swing_amp * std::sin(static_cast<double>(r->swing_omega) * t)),
                  r->wind[1], r->wind[2]};
    std::memcpy(r->groom->wind, w, sizeof(w));
    S->active.push_back(r->groom);
    S->advancing.push_back(r);
    st.point_substeps += static_cast<uint64_t>(r->nstrands) * r->strand.points_per_strand * r->sim.substeps;
  }
  if (!S->active.empty()) {
    hs_status bs = batch_update(S->ctx, S->active.data(), static_cast<uint32_t>(S->active.size()), dt);
    if (bs != HS_OK) return bs;
  }
  e = cudaStreamSynchronize(S->ctx->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hs_server_tick");
  for (Request* r : S->advancing) ++r->frames_done;
  st.advanced = static_cast<uint32_t>(S->active.size());
  st.queued = static_cast<uint32_t>(S->queue.size());
  st.resident_bytes = S->pool.used();
  st.tick_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (out) *out = st;
  return HS_OK;
}

// A request whose inputs the caller may still change: queued, or resident
// with frames to go.
static hs_status live_request(hs_server* S, uint64_t ticket, const char* what, Request** out) {
  if (!S) return fail(HS_ERR_INVALID_ARG, "%s: null server", what);
  auto it = S->by_ticket.find(ticket);
  if (it == S->by_ticket.end() || it->second->state == HS_REQ_DONE || it->second->frames_done >= it->second->frames)
    return fail(HS_ERR_INVALID_ARG, "%s: request %llu is neither queued nor running", what,
                static_cast<unsigned long long>(ticket));
  *out = it->second;
  return HS_OK;
}

HS_API hs_status hs_server_set_spheres(hs_server* S, uint64_t ticket, const float* xyzr, uint32_t n) {
  Request* r = nullptr;
  hs_status st = live_request(S, ticket, "hs_server_set_spheres", &r);
  if (st != HS_OK) return st;
  if (n > 0 && !xyzr) return fail(HS_ERR_INVALID_ARG, "hs_server_set_spheres: null spheres");
  if (r->groom) return set_spheres(r->groom, xyzr, n);
  // Queued: validated now, applied at admission.
  if (n > HS_MAX_SPHERES) return fail(HS_ERR_INVALID_ARG, "hs_server_set_spheres: %u spheres > %d", n, HS_MAX_SPHERES);
  for (uint32_t k = 0; k < 4 * n; ++k)
    if (!std::isfinite(xyzr[k]) || (k % 4 == 3 && xyzr[k] < 0.0f))
      return fail(HS_ERR_INVALID_ARG, "hs_server_set_spheres: sphere %u is invalid", k / 4);
  r->spheres.assign(xyzr, xyzr + 4 * static_cast<size_t>(n));
  return HS_OK;
}

HS_API hs_status hs_server_set_root_transform(hs_server* S, uint64_t ticket, const float m[16]) {
  Request* r = nullptr;
  hs_status st = live_request(S, ticket, "hs_server_set_root_transform", &r);
  if (st != HS_OK) return st;
  if (r->sim.root_mode != HS_ROOT_RIGID)
    return fail(HS_ERR_UNSUPPORTED, "hs_server_set_root_transform: request %llu does not have rigid roots",
                static_cast<unsigned long long>(ticket));
  if (!m) return fail(HS_ERR_INVALID_ARG, "hs_server_set_root_transform: null matrix");
  for (int c = 0; c < 16; ++c)
    if (!std::isfinite(m[c])) return fail(HS_ERR_INVALID_ARG, "hs_server_set_root_transform: non-finite entry %d", c);
  std::memcpy(r->m, m, sizeof(r->m));
  if (r->groom) std::memcpy(r->groom->m, m, sizeof(r->m));
  return HS_OK;
}

HS_API hs_status hs_server_set_bone_matrices(hs_server* S, uint64_t ticket, const float* m, uint32_t nbones) {
  Request* r = nullptr;
  hs_status st = live_request(S, ticket, "hs_server_set_bone_matrices", &r);
  if (st != HS_OK) return st;
  if (r->sim.root_mode != HS_ROOT_SKINNED)
    return fail(HS_ERR_UNSUPPORTED, "hs_server_set_bone_matrices: request %llu does not have skinned roots",
                static_cast<unsigned long long>(ticket));
  if ((nbones > 0 && !m) || nbones > HS_MAX_BONES)
    return fail(HS_ERR_INVALID_ARG, "hs_server_set_bone_matrices: %u bones (at most %d)", nbones, HS_MAX_BONES);
  float dq[8 * HS_MAX_BONES] = {};
  for (uint32_t b = 0; b < nbones; ++b) {
    const float* mb = m + 16 * static_cast<size_t>(b);
    for (int k = 0; k < 16; ++k)
      if (!std::isfinite(mb[k])) return fail(HS_ERR_INVALID_ARG, "hs_server_set_bone_matrices: bone %u non-finite", b);
    matrix_to_dual_quat(mb, dq + 8 * b);
  }
  if (r->groom) {
    st = hs_set_bone_dual_quats(r->groom, dq, nbones);
    if (st != HS_OK) return st;
  }
  std::memcpy(r->dq, dq, sizeof(dq));
  r->nbones = nbones;
  r->has_palette = true;
  return HS_OK;
}

HS_API hs_status hs_server_poll(hs_server* S, uint64_t ticket, uint32_t* out_state, uint32_t* out_frames_done) {
  if (!S) return fail(HS_ERR_INVALID_ARG, "hs_server_poll: null server");
  auto it = S->by_ticket.find(ticket);
  if (it == S->by_ticket.end()) {
    if (out_state) *out_state = HS_REQ_GONE;
    if (out_frames_done) *out_frames_done = 0;
    return HS_OK;
  }
  Request* r = it->second;
  // A groom that has done its frames is DONE from the caller's view even
  // before the next tick retires it.
  uint32_t state = r->state;
  if (state == HS_REQ_RESIDENT && r->frames_done >= r->frames) state = r->keep ? HS_REQ_DONE : HS_REQ_GONE;
  if (out_state) *out_state = state;
  if (out_frames_done) *out_frames_done = r->frames_done;
  return HS_OK;
}

HS_API hs_status hs_server_collect(hs_server* S, uint64_t ticket, float* pos, float* vel, size_t capacity_floats) {
  if (!S) return fail(HS_ERR_INVALID_ARG, "hs_server_collect: null server");
  HS_ON_DEVICE(S->ctx, "hs_server_collect");
  auto it = S->by_ticket.find(ticket);
  if (it == S->by_ticket.end()) return fail(HS_ERR_INVALID_ARG, "hs_server_collect: unknown ticket");
  Request* r = it->second;
  if (!r->keep || r->frames_done < r->frames)
    return fail(HS_ERR_NOT_INITIALIZED, "hs_server_collect: request %llu has no result yet",
                static_cast<unsigned long long>(ticket));
  hs_status st = HS_OK;
  if (pos) st = hs_readback(r->groom, pos, capacity_floats);
  if (st == HS_OK && vel) st = hs_readback_velocities(r->groom, vel, capacity_floats);
  if (st != HS_OK) return st;
  S->resident.erase(std::remove(S->resident.begin(), S->resident.end(), r), S->resident.end());
  release_request(S, r);
  S->by_ticket.erase(it);
  delete r;
  return HS_OK;
}

}  // extern "C"
