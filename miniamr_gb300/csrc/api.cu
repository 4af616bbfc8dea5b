// Host side of the GB300 library: the mamr_* C ABI (include/miniamr_gb300.h).
//
// A context owns one zero-filled cell pool on the current device, a CUDA
// stream, the per-direction exchange task lists derived from the mesh, and
// small device buffers for checksum results.  Every entry point validates
// its arguments on the host, queues kernels on the context's stream and
// returns a status; nothing here exits the process.
#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <tuple>
#include <new>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mamr_internal.h"
#include "batched.h"
#include "mark_geometry.h"
#include "segments.h"

using namespace mamr;

static thread_local char g_err[512];

static int fail(int code, const char *fmt, ...)
{
   va_list ap;
   va_start(ap, fmt);
   vsnprintf(g_err, sizeof(g_err), fmt, ap);
   va_end(ap);
   return code;
}

extern "C" const char *mamr_last_error(void) { return g_err; }

// How the AMR driver (amr_driver.cpp) records its own failures.
extern "C" int mamr_driver_fail(int code, const char *msg)
{
   return fail(code, "%s", msg);
}

int mamr::report_error(int code, const char *fmt, ...)
{
   va_list ap;
   va_start(ap, fmt);
   vsnprintf(g_err, sizeof(g_err), fmt, ap);
   va_end(ap);
   return code;
}

#define CUDA_TRY(x)                                                         \
   do {                                                                     \
      cudaError_t e_ = (x);                                                 \
      if (e_ != cudaSuccess)                                                \
         return fail(MAMR_ECUDA, "%s: %s", #x, cudaGetErrorString(e_));     \
   } while (0)

#define LAUNCH_TRY(ctx, x)                                                  \
   do {                                                                     \
      int n_ = (x);                                                         \
      if (n_ < 0)                                                           \
         return fail(MAMR_ECUDA, "launch %s: %s", #x,                      \
                     cudaGetErrorString(cudaGetLastError()));               \
      (ctx)->launches += n_;                                                \
   } while (0)

namespace {

// Growable device buffer.
struct DevBuf {
   void *p = nullptr;
   size_t cap = 0;
   cudaError_t ensure(size_t bytes)
   {
      if (bytes <= cap)
         return cudaSuccess;
      if (p)
         cudaFree(p);
      p = nullptr;
      cap = 0;
      size_t want = bytes + bytes / 4 + 256;
      cudaError_t e = cudaMalloc(&p, want);
      if (e == cudaSuccess)
         cap = want;
      return e;
   }
   void release()
   {
      if (p)
         cudaFree(p);
      p = nullptr;
      cap = 0;
   }
};

const int kPerm[6][3] = { {0, 1, 2}, {1, 2, 0}, {2, 0, 1},
                          {0, 2, 1}, {1, 0, 2}, {2, 1, 0} };

}  // namespace

namespace mamr {
struct BatchedState {
   DevBuf items, partials, sums, acc, chain, pencils, bad;
   DevBuf csflags;             // FP32: per checksum stage, 1 + V miss words
                               // and the fallback's counter
   DevBuf zf[2];               // the warp-per-block kernel's z-face arrays
                               // (stage q writes zf[q & 1])
   DevBuf recipes, keep;       // 27-point edge/corner recipes (multi-level)
                               // and the blocks' keep masks
   bool has_recipes = false;
   BItem *h_items = nullptr;   // pinned staging of the item upload
   size_t h_cap = 0;           // its capacity in items
   int n = 0;
   bool valid = false;
   bool single_level = false;
   int grid = 0;
   int n_pencils = 0;     // > 0: the pencil kernel applies
};
void batched_destroy(BatchedState *b)
{
   if (!b)
      return;
   b->items.release(); b->partials.release(); b->sums.release();
   b->acc.release(); b->chain.release(); b->pencils.release();
   b->bad.release(); b->csflags.release(); b->recipes.release();
   b->zf[0].release(); b->zf[1].release();
   b->keep.release();
   if (b->h_items)
      cudaFreeHost(b->h_items);
   delete b;
}
void batched_mesh_changed(BatchedState *b)
{
   if (b)
      b->valid = false;
}
}  // namespace mamr

struct mamr_ctx {
   mamr_config cfg;
   Geom g;
   bool fp32;
   int device;
   cudaStream_t stream;
   void *pool;             // current pool
   size_t pool_bytes;
   void *pool_alt;         // second pool for the batched ping-pong (lazy)
   size_t pool_shift;      // bytes both pools start past their allocations
   // The mesh as mamr_set_mesh last took it: a view of one of two pinned
   // host buffers, which the mesh's upload to d_mesh reads; the next mesh
   // goes into the other one (once that one's upload has run).
   struct MeshView {
      const mamr_block *p = nullptr;
      size_t n = 0;
      size_t size() const { return n; }
      const mamr_block &operator[](size_t i) const { return p[i]; }
      const mamr_block *begin() const { return p; }
      const mamr_block *end() const { return p + n; }
   };
   MeshView mesh;
   struct MeshBuf {
      mamr_block *p = nullptr;
      size_t cap = 0;
      cudaEvent_t ev = nullptr;
      bool pending = false;
   };
   MeshBuf hmesh[2];
   int hmesh_cur = 0;
   std::vector<int32_t> slot_pos;   // slot -> index in mesh or -1
   DevBuf d_slots;                  // sorted slots
   DevBuf d_mesh, d_slot_pos;       // device copies of mesh and slot_pos
   DevBuf d_tasks[3];
   DirTasks tasks[3];
   bool tasks_dirty = true;         // tasks[] not built for the mesh yet
   DevBuf d_partials, d_jobs, d_stage, d_stage_slots, d_sums;
   DevBuf d_xfer, d_xfer_slots;      // staging copies for split/consolidate
   DevBuf d_csflags;                // FP32 checksum miss words (plain path)
   unsigned long long *d_acc;       // 2 words: fixed-point accumulator
   double *d_sum;                   // FP64 checksum result
   unsigned *d_err;                 // device error word
   void *h_pinned;                  // 64 bytes of pinned host memory
   long long launches;
   int hw_slots;                    // 1 + highest slot ever holding data
   mamr::BatchedState *batched;
   mamr_work_par work{};            // --stencil 0 coefficients
   bool work_set = false;
   DevBuf d_work;                   // --stencil 0 work values
   DevBuf d_mark;                   // refinement marking lists and flags
   // the plain path's z-face cache (mamr_internal.h: zcache_at) and, per
   // variable, whether it holds what the pool holds: set by a plain
   // stencil of the variable, cleared by anything else that changes
   // interior cells or the mesh
   DevBuf d_zc;
   std::vector<char> zc_ok;
   // FP64 checksums of every variable, computed together on the first
   // mamr_check_sum after the pool or the mesh last changed (gen counts
   // those changes)
   unsigned long long gen = 0, cs_gen = ~0ull;
   std::vector<double> cs_host;
   DevBuf d_cs;
   int tune_force = -1;             // forced launch-shape candidate
   int tune_last = -1, tune_n = 0;  // last batched run's choice / count
   mamr::StageShape tune_shape;
   // pinned host staging of the copies mamr_split, mamr_consolidate and
   // mamr_set_mesh queue without waiting for them: a ring whose slots are
   // taken again once the copies from them have run (an event each)
   struct HostStage {
      void *p = nullptr;
      size_t cap = 0;
      cudaEvent_t ev = nullptr;
      bool pending = false;
   };
   static constexpr int kHostStages = 8;
   HostStage hstage[kHostStages];
   int hstage_next = 0;
   // the batched path's z-face arrays across runs: zface_live is the array
   // (0 or 1) that holds the k = 1 and k = nz planes of every slot
   // zface_ok marks, as the pool holds them -- written by the last stage
   // of a run with the warp-per-block or tile kernel and, while live, by
   // splits and consolidations for the blocks they write -- or -1 when
   // none does; a run's first stage then reads its z ghosts from there
   int zface_live = -1;
   std::vector<char> zface_ok;
};

static size_t elem_size(const mamr_ctx *c) { return c->fp32 ? 4 : 8; }

// Host threads (OpenMP) of the checks and copies over long block lists.
[[maybe_unused]] constexpr int kHostThreads = 4;

// The next slot of the host staging ring, at least `bytes` long, once the
// copies queued from it before have run; null on a CUDA error (*e).
static void *host_stage_take(mamr_ctx *c, size_t bytes, int *slot,
                             cudaError_t *e)
{
   *slot = c->hstage_next;
   c->hstage_next = (c->hstage_next + 1) % mamr_ctx::kHostStages;
   mamr_ctx::HostStage &h = c->hstage[*slot];
   *e = cudaSuccess;
   if (h.pending) {
      h.pending = false;
      if ((*e = cudaEventSynchronize(h.ev)) != cudaSuccess)
         return nullptr;
   }
   if (!h.ev &&
       (*e = cudaEventCreateWithFlags(&h.ev, cudaEventDisableTiming)) !=
          cudaSuccess)
      return nullptr;
   if (h.cap < bytes) {
      if (h.p)
         cudaFreeHost(h.p);
      h.p = nullptr;
      h.cap = 0;
      const size_t want = bytes + bytes / 4 + 4096;
      if ((*e = cudaMallocHost(&h.p, want)) != cudaSuccess)
         return nullptr;
      h.cap = want;
   }
   return h.p;
}

// The copies from ring slot `slot` are queued: the slot is taken again
// after they have run.
static cudaError_t host_stage_queued(mamr_ctx *c, int slot)
{
   mamr_ctx::HostStage &h = c->hstage[slot];
   const cudaError_t e = cudaEventRecord(h.ev, c->stream);
   h.pending = e == cudaSuccess;
   return e;
}

// Where a pool starts past its (256-byte aligned) allocation: so that the
// interior row (1, 1) of every block-variable -- each i-plane's interior
// rows are one contiguous run -- starts a 128-byte line, which block-
// variable strides of whole lines then keep for all of them (16^3 FP32:
// 64 bytes, and every interior i-plane is 8 whole lines instead of 9
// partial ones; 8^3 FP32: 32 bytes, every other plane whole; 8^3 FP64: 64;
// 16^3 FP64: 0).  A multiple of 16 bytes, which every vector access and
// tensor copy of the pool needs.
static size_t pool_shift(const Geom &g, size_t es)
{
   const size_t off = ((size_t) g.Y + 1) * (size_t) g.nz * es;
   return ((128 - off % 128) % 128) & ~(size_t) 15;
}

// A pool of c->pool_bytes past c->pool_shift bytes of its allocation, zero
// filled (queued on the context's stream).
static cudaError_t pool_alloc(mamr_ctx *c, void **pool)
{
   char *base = nullptr;
   const size_t bytes = c->pool_bytes + c->pool_shift;
   cudaError_t e = cudaMalloc((void **) &base, bytes);
   if (e == cudaSuccess)
      e = cudaMemsetAsync(base, 0, bytes, c->stream);
   if (e != cudaSuccess) {
      if (base)
         cudaFree(base);
      return e;
   }
   *pool = base + c->pool_shift;
   return cudaSuccess;
}

static void pool_free(mamr_ctx *c, void *pool)
{
   if (pool)
      cudaFree((char *) pool - c->pool_shift);
}

// The z-face cache: dropped whenever interior cells or the mesh change
// other than through a plain stencil; the buffer a plain stencil writes
// (allocated on first use; null if it cannot be, and the stencil then
// writes none).
static void zcache_drop(mamr_ctx *c)
{
   std::fill(c->zc_ok.begin(), c->zc_ok.end(), 0);
}
// The live z-face array (for splits and consolidations to store the
// planes of the blocks they write), or null.
static void *zface_live_array(mamr_ctx *c)
{
   if (c->zface_live < 0 || !c->batched)
      return nullptr;
   return c->batched->zf[c->zface_live].p;
}

static void *zcache_for_stencil(mamr_ctx *c)
{
   if (!c->d_zc.p) {
      const size_t bytes =
         zcache_elems(c->g, c->cfg.max_blocks) * elem_size(c);
      if (c->d_zc.ensure(bytes) != cudaSuccess) {
         cudaGetLastError();
         c->d_zc.release();
         return nullptr;
      }
      c->zc_ok.assign(c->cfg.num_vars, 0);
   }
   return c->d_zc.p;
}


static int check_error_word(mamr_ctx *c)
{
   unsigned h = 0;
   CUDA_TRY(cudaMemcpyAsync(&h, c->d_err, sizeof(h), cudaMemcpyDeviceToHost,
                            c->stream));
   CUDA_TRY(cudaStreamSynchronize(c->stream));
   if (h) {
      CUDA_TRY(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
      if (h & ERR_FIXED_RANGE)
         return fail(MAMR_EDEVICE, "a cell is outside the FP32 checksum's "
                     "fixed-point range (|v| < 1024, finite)");
      if (h & ERR_MARK)
         return fail(MAMR_EDEVICE, "refinement marking did not settle");
      if (h & ERR_WAIT)
         return fail(MAMR_EDEVICE, "a stage kernel's wait for its tensor "
                     "copies ran out (results of the run are invalid)");
      return fail(MAMR_EDEVICE, "device error word 0x%x", h);
   }
   return MAMR_OK;
}

extern "C" int mamr_create(const mamr_config *cfg, mamr_ctx **out)
{
   if (!cfg || !out)
      return fail(MAMR_EINVAL, "null argument");
   *out = nullptr;
   if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2 || cfg->nx % 2 ||
       cfg->ny % 2 || cfg->nz % 2)
      return fail(MAMR_EINVAL, "block sizes must be even and >= 2");
   if (cfg->num_vars < 1 || cfg->num_vars > 65535 || cfg->max_blocks < 1)
      return fail(MAMR_EINVAL, "num_vars must be in 1..65535 and "
                  "max_blocks >= 1");
   if (cfg->stencil != 0 && cfg->stencil != 7 && cfg->stencil != 27)
      return fail(MAMR_EUNSUP, "stencil %d not supported", cfg->stencil);
   if (cfg->stencil == 0 && cfg->dtype != MAMR_FP64)
      return fail(MAMR_EUNSUP, "stencil 0 runs on FP64 pools only");
   if (cfg->stencil == 0 &&
       (cfg->num_vars < 8 || cfg->num_vars / 4 > MAMR_WORK_MAX_MAT))
      return fail(MAMR_EINVAL, "stencil 0 needs 8 <= num_vars <= %d",
                  4 * MAMR_WORK_MAX_MAT + 3);
   if (cfg->code < 0 || cfg->code > 2)
      return fail(MAMR_EUNSUP, "code %d not supported", cfg->code);
   if (cfg->dtype != MAMR_FP64 && cfg->dtype != MAMR_FP32)
      return fail(MAMR_EINVAL, "bad dtype");
   for (int r = 0; r < 7; r++)
      if (cfg->reserved[r])
         return fail(MAMR_EINVAL, "reserved fields must be zero");

   mamr_ctx *c = new (std::nothrow) mamr_ctx();
   if (!c)
      return fail(MAMR_ENOMEM, "host allocation");
   c->cfg = *cfg;
   c->fp32 = cfg->dtype == MAMR_FP32;
   Geom &g = c->g;
   g.nx = cfg->nx; g.ny = cfg->ny; g.nz = cfg->nz; g.V = cfg->num_vars;
   g.X = g.nx + 2; g.Y = g.ny + 2; g.Z = g.nz + 2;
   // split layout: dense interior rows, then the two k-ghost planes; a
   // block-variable takes whole 128-byte lines (and the pool's start,
   // pool_shift, puts its interior rows on line boundaries)
   const int line = 128 / (int) elem_size(c);
   g.Zp = g.Z;
   g.koff = 0;
   g.kplane = (long long) g.X * g.Y * g.nz;
   g.bv = ((g.kplane + 2LL * g.X * g.Y + line - 1) / line) * line;
   if (!plain_stencil_fits(g, elem_size(c))) {
      delete c;
      return fail(MAMR_EUNSUP, "blocks of %d x %d cells per i-plane do not "
                  "fit the stencil's three-plane ring (%zu KiB)", g.Y, g.Z,
                  kPlainRingBytes / 1024);
   }
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e == cudaSuccess)
      e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
   c->device = dev;
   c->pool_bytes = (size_t) cfg->max_blocks * g.V * g.bv * elem_size(c);
   c->pool_shift = pool_shift(g, elem_size(c));
   if (e == cudaSuccess)
      e = pool_alloc(c, &c->pool);
   if (e == cudaSuccess)
      e = cudaMalloc((void **) &c->d_acc, 64);
   if (e == cudaSuccess)
      e = cudaMalloc((void **) &c->d_sum, 64);
   if (e == cudaSuccess)
      e = cudaMalloc((void **) &c->d_err, 64);
   if (e == cudaSuccess)
      e = cudaMemsetAsync(c->d_err, 0, 64, c->stream);
   if (e == cudaSuccess)
      e = cudaMallocHost(&c->h_pinned, 64);
   if (e == cudaSuccess)
      e = cudaStreamSynchronize(c->stream);
   if (e != cudaSuccess) {
      int code = (e == cudaErrorMemoryAllocation) ? MAMR_ENOMEM : MAMR_ECUDA;
      mamr_destroy(c);
      cudaGetLastError();
      return fail(code, "mamr_create: %s", cudaGetErrorString(e));
   }
   c->slot_pos.assign(cfg->max_blocks, -1);
   c->zface_ok.assign(cfg->max_blocks, 0);
   *out = c;
   return MAMR_OK;
}

extern "C" int mamr_destroy(mamr_ctx *c)
{
   if (!c)
      return MAMR_OK;
   if (c->stream)
      cudaStreamSynchronize(c->stream);
   mamr::batched_destroy(c->batched);
   pool_free(c, c->pool);
   pool_free(c, c->pool_alt);
   for (mamr_ctx::MeshBuf &h : c->hmesh) {
      if (h.ev)
         cudaEventDestroy(h.ev);
      if (h.p)
         cudaFreeHost(h.p);
   }
   for (mamr_ctx::HostStage &h : c->hstage) {
      if (h.ev)
         cudaEventDestroy(h.ev);
      if (h.p)
         cudaFreeHost(h.p);
   }
   for (auto &b : c->d_tasks) b.release();
   c->d_slots.release(); c->d_partials.release(); c->d_jobs.release();
   c->d_stage.release(); c->d_stage_slots.release(); c->d_sums.release();
   c->d_xfer.release(); c->d_xfer_slots.release(); c->d_work.release();
   c->d_mark.release(); c->d_cs.release(); c->d_zc.release();
   c->d_mesh.release(); c->d_slot_pos.release(); c->d_csflags.release();
   if (c->d_acc) cudaFree(c->d_acc);
   if (c->d_sum) cudaFree(c->d_sum);
   if (c->d_err) cudaFree(c->d_err);
   if (c->h_pinned) cudaFreeHost(c->h_pinned);
   if (c->stream) cudaStreamDestroy(c->stream);
   delete c;
   return MAMR_OK;
}

extern "C" int mamr_stream(mamr_ctx *c, void **stream)
{
   if (!c || !stream)
      return fail(MAMR_EINVAL, "null argument");
   *stream = (void *) c->stream;
   return MAMR_OK;
}

extern "C" int mamr_sync(mamr_ctx *c)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   CUDA_TRY(cudaStreamSynchronize(c->stream));
   return check_error_word(c);
}

extern "C" int mamr_launch_count(mamr_ctx *c, int64_t *count)
{
   if (!c || !count)
      return fail(MAMR_EINVAL, "null argument");
   *count = c->launches;
   return MAMR_OK;
}

static bool slot_ok(const mamr_ctx *c, int32_t s)
{
   return s >= 0 && s < c->cfg.max_blocks;
}

// Host buffers that are not pinned move through a bounded device staging
// area.
static const size_t kStageBytes = 256u << 20;

static int transfer(mamr_ctx *c, const int32_t *slots, int32_t n,
                    double *host, bool up)
{
   if (n < 0 || (n && (!slots || !host)))
      return fail(MAMR_EINVAL, "bad transfer arguments");
   for (int32_t b = 0; b < n; b++)
      if (!slot_ok(c, slots[b]))
         return fail(MAMR_EINVAL, "slot %d out of range", slots[b]);
   if (up)
      for (int32_t b = 0; b < n; b++)
         c->hw_slots = std::max(c->hw_slots, slots[b] + 1);
   const Geom &g = c->g;
   const size_t per_block = (size_t) g.V * g.X * g.Y * g.Z;
   // Pinned host memory the device can address: one launch reads (or
   // writes) it in place over the host link -- no staging copy and no
   // synchronisation per chunk.
   cudaPointerAttributes pa;
   if (n && cudaPointerGetAttributes(&pa, host) == cudaSuccess &&
       pa.type == cudaMemoryTypeHost && pa.devicePointer &&
       !(reinterpret_cast<uintptr_t>(pa.devicePointer) & 15)) {
      double *dh = static_cast<double *>(pa.devicePointer);
      CUDA_TRY(c->d_stage_slots.ensure(sizeof(int32_t) * n));
      CUDA_TRY(cudaMemcpyAsync(c->d_stage_slots.p, slots, sizeof(int32_t) * n,
                               cudaMemcpyHostToDevice, c->stream));
      const int32_t *ds = (const int32_t *) c->d_stage_slots.p;
      if (up && c->fp32)
         LAUNCH_TRY(c, launch_upload((float *) c->pool, g, ds, n, dh,
                                     c->stream));
      else if (up)
         LAUNCH_TRY(c, launch_upload((double *) c->pool, g, ds, n, dh,
                                     c->stream));
      else if (c->fp32)
         LAUNCH_TRY(c, launch_download((const float *) c->pool, g, ds, n, dh,
                                       c->stream));
      else
         LAUNCH_TRY(c, launch_download((const double *) c->pool, g, ds, n, dh,
                                       c->stream));
      CUDA_TRY(cudaStreamSynchronize(c->stream));
      return MAMR_OK;
   }
   cudaGetLastError();
   int32_t chunk = (int32_t) std::max<size_t>(1, kStageBytes /
                                              (per_block * sizeof(double)));
   CUDA_TRY(c->d_stage.ensure(std::min<size_t>(n, chunk) * per_block *
                              sizeof(double)));
   CUDA_TRY(c->d_stage_slots.ensure(sizeof(int32_t) * std::max(1, chunk)));
   for (int32_t b0 = 0; b0 < n; b0 += chunk) {
      int32_t m = std::min(chunk, n - b0);
      double *h = host + (size_t) b0 * per_block;
      CUDA_TRY(cudaMemcpyAsync(c->d_stage_slots.p, slots + b0,
                               sizeof(int32_t) * m, cudaMemcpyHostToDevice,
                               c->stream));
      if (up) {
         CUDA_TRY(cudaMemcpyAsync(c->d_stage.p, h,
                                  sizeof(double) * per_block * m,
                                  cudaMemcpyHostToDevice, c->stream));
         if (c->fp32)
            LAUNCH_TRY(c, launch_upload((float *) c->pool, g,
                                        (const int32_t *) c->d_stage_slots.p,
                                        m, (const double *) c->d_stage.p,
                                        c->stream));
         else
            LAUNCH_TRY(c, launch_upload((double *) c->pool, g,
                                        (const int32_t *) c->d_stage_slots.p,
                                        m, (const double *) c->d_stage.p,
                                        c->stream));
      } else {
         if (c->fp32)
            LAUNCH_TRY(c, launch_download((const float *) c->pool, g,
                                          (const int32_t *) c->d_stage_slots.p,
                                          m, (double *) c->d_stage.p,
                                          c->stream));
         else
            LAUNCH_TRY(c, launch_download((const double *) c->pool, g,
                                          (const int32_t *) c->d_stage_slots.p,
                                          m, (double *) c->d_stage.p,
                                          c->stream));
         CUDA_TRY(cudaMemcpyAsync(h, c->d_stage.p,
                                  sizeof(double) * per_block * m,
                                  cudaMemcpyDeviceToHost, c->stream));
      }
      CUDA_TRY(cudaStreamSynchronize(c->stream));
   }
   return MAMR_OK;
}

extern "C" int mamr_upload_blocks(mamr_ctx *c, const int32_t *slots,
                                  int32_t n, const double *host)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   c->gen++;
   zcache_drop(c);
   c->zface_live = -1;
   return transfer(c, slots, n, const_cast<double *>(host), true);
}

extern "C" int mamr_download_blocks(mamr_ctx *c, const int32_t *slots,
                                    int32_t n, double *host)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   return transfer(c, slots, n, host, false);
}

// Per-block checks of mamr_set_mesh that need no other block: the slot
// and, on every face, the neighbour level and the neighbour slots the face
// uses.
static bool mesh_block_ok(const mamr_ctx *c, const mamr_block &bp)
{
   if (!slot_ok(c, bp.slot))
      return false;
   for (int l = 0; l < 6; l++) {
      const int nl = bp.nei_level[l];
      if (nl == -2)
         continue;
      if (nl != bp.level && nl != bp.level + 1 && nl != bp.level - 1)
         return false;
      const int cnt = nl == bp.level + 1 ? 4 : 1;
      for (int q = 0; q < cnt; q++)
         if (!slot_ok(c, bp.nei[l][q >> 1][q & 1]))
            return false;
   }
   return true;
}

// mamr_set_mesh's checks and copies for a long mesh on kHostThreads
// threads: each slot's position claimed by an atomic exchange (a slot
// listed twice finds it taken), the blocks copied into dst and their slots
// into hs.  False on any failure, after which the serial checks name it.
static bool set_mesh_parallel(const mamr_ctx *c, const mamr_block *blocks,
                              int32_t n, int32_t *pos, mamr_block *dst,
                              int32_t *hs, int *hw)
{
   const int32_t cap = c->cfg.max_blocks;
   int bad = 0, top = 0;
#pragma omp parallel num_threads(kHostThreads) reduction(| : bad) \
   reduction(max : top)
   {
#pragma omp for schedule(static)
      for (int32_t b = 0; b < n; b++) {
         const mamr_block &bp = blocks[b];
         dst[b] = bp;
         hs[b] = bp.slot;
         int32_t none = -1;
         if (!mesh_block_ok(c, bp) ||
             !__atomic_compare_exchange_n(&pos[bp.slot], &none, b, false,
                                          __ATOMIC_RELAXED, __ATOMIC_RELAXED))
            bad = 1;
         else
            top = std::max(top, bp.slot + 1);
      }
      // every listed neighbour active (slots checked again: a block that
      // failed above may list any value)
#pragma omp for schedule(static)
      for (int32_t b = 0; b < n; b++) {
         const mamr_block &bp = blocks[b];
         for (int l = 0; l < 6; l++) {
            const int nl = bp.nei_level[l];
            if (nl == -2)
               continue;
            const int cnt = nl == bp.level + 1 ? 4 : 1;
            for (int q = 0; q < cnt; q++) {
               const int m = bp.nei[l][q >> 1][q & 1];
               if (m < 0 || m >= cap || pos[m] < 0)
                  bad = 1;
            }
         }
      }
   }
   *hw = top;
   return !bad;
}

// The mesh: checked (the reference's misconnected-block errors,
// ref/comm.c:198-201), its slots, blocks and slot positions uploaded
// (queued); the face exchange's task lists follow on its first call
// (build_tasks).  The blocks are kept in the pinned buffer the upload reads.
extern "C" int mamr_set_mesh(mamr_ctx *c, const mamr_block *blocks,
                             int32_t n)
{
   if (!c || n < 0 || (n && !blocks))
      return fail(MAMR_EINVAL, "bad mesh arguments");
   if (n > c->cfg.max_blocks)
      return fail(MAMR_EINVAL, "%d blocks exceed max_blocks", n);
   // the pinned buffer the current mesh is not in, once its last upload
   // has run
   const int k = 1 - c->hmesh_cur;
   mamr_ctx::MeshBuf &hm = c->hmesh[k];
   if (hm.pending) {
      hm.pending = false;
      CUDA_TRY(cudaEventSynchronize(hm.ev));
   }
   if (!hm.ev)
      CUDA_TRY(cudaEventCreateWithFlags(&hm.ev, cudaEventDisableTiming));
   if (hm.cap < (size_t) std::max(1, n)) {
      if (hm.p)
         cudaFreeHost(hm.p);
      hm.p = nullptr;
      hm.cap = 0;
      const size_t want = std::min<size_t>(
         (size_t) std::max(1, n) * 5 / 4 + 64, c->cfg.max_blocks + (size_t) 1);
      CUDA_TRY(cudaMallocHost((void **) &hm.p, sizeof(mamr_block) * want));
      hm.cap = want;
   }
   // slots and slot positions through the pinned ring
   const size_t bs = sizeof(int32_t) * (size_t) n;
   const size_t bp = sizeof(int32_t) * (size_t) c->cfg.max_blocks;
   const size_t op = (bs + 15) & ~(size_t) 15;
   int slot = 0;
   cudaError_t e;
   char *h = (char *) host_stage_take(c, op + bp + 16, &slot, &e);
   if (!h)
      return fail(MAMR_ECUDA, "host staging: %s", cudaGetErrorString(e));
   int32_t *hs = reinterpret_cast<int32_t *>(h);
   std::vector<int32_t> pos(c->cfg.max_blocks, -1);
   int hw = 0;
   bool done = n >= 4096 &&
               set_mesh_parallel(c, blocks, n, pos.data(), hm.p, hs, &hw);
   if (!done) {
      std::fill(pos.begin(), pos.end(), -1);
      for (int32_t b = 0; b < n; b++) {
         const mamr_block &bp = blocks[b];
         if (!slot_ok(c, bp.slot))
            return fail(MAMR_EINVAL, "block %d: slot %d out of range", b,
                        bp.slot);
         if (pos[bp.slot] >= 0)
            return fail(MAMR_EINVAL, "slot %d listed twice", bp.slot);
         pos[bp.slot] = b;
         for (int l = 0; l < 6; l++) {
            int nl = bp.nei_level[l];
            if (nl == -2)
               continue;
            if (nl != bp.level && nl != bp.level + 1 && nl != bp.level - 1)
               return fail(MAMR_EMESH, "misconnected block (slot %d face %d)",
                           bp.slot, l);
            for (int i = 0; i < 2; i++)
               for (int j = 0; j < 2; j++)
                  if ((nl == bp.level + 1 || (i == 0 && j == 0)) &&
                      !slot_ok(c, bp.nei[l][i][j]))
                     return fail(MAMR_EMESH, "misconnected block (slot %d "
                                 "face %d nei %d)", bp.slot, l,
                                 bp.nei[l][i][j]);
         }
      }
      // every listed neighbour must be active, whichever of the pair
      // visits the face (the batched path reads each block's own list)
      for (int32_t in = 0; in < n; in++) {
         const mamr_block &bp = blocks[in];
         for (int l = 0; l < 6; l++) {
            const int nl = bp.nei_level[l];
            if (nl == -2)
               continue;
            const int cnt = nl == bp.level + 1 ? 4 : 1;
            for (int q = 0; q < cnt; q++) {
               const int m = bp.nei[l][q >> 1][q & 1];
               if (pos[m] < 0)
                  return fail(MAMR_EMESH, "neighbour slot %d not active", m);
            }
         }
      }
      for (int32_t b = 0; b < n; b++) {
         hs[b] = blocks[b].slot;
         hw = std::max(hw, blocks[b].slot + 1);
      }
      if (n)
         memcpy(hm.p, blocks, sizeof(mamr_block) * n);
   }
   c->gen++;
   zcache_drop(c);
   memcpy(h + op, pos.data(), bp);
   // sorted slots now; the face exchange's task lists when it first runs
   // on this mesh (build_tasks), since a batched run never needs them
   CUDA_TRY(c->d_slots.ensure(sizeof(int32_t) * std::max(1, n)));
   c->tasks_dirty = true;
   CUDA_TRY(c->d_partials.ensure(sizeof(double) * std::max(1, n) *
                                 c->cfg.num_vars));
   // the mesh on the device, for the batched path's descriptor build
   CUDA_TRY(c->d_mesh.ensure(sizeof(mamr_block) * std::max(1, n)));
   CUDA_TRY(c->d_slot_pos.ensure(bp));
   if (n) {
      CUDA_TRY(cudaMemcpyAsync(c->d_slots.p, h, bs, cudaMemcpyHostToDevice,
                               c->stream));
      CUDA_TRY(cudaMemcpyAsync(c->d_mesh.p, hm.p, sizeof(mamr_block) * n,
                               cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(cudaEventRecord(hm.ev, c->stream));
      hm.pending = true;
   }
   CUDA_TRY(cudaMemcpyAsync(c->d_slot_pos.p, h + op, bp,
                            cudaMemcpyHostToDevice, c->stream));
   CUDA_TRY(host_stage_queued(c, slot));
   c->mesh.p = hm.p;
   c->mesh.n = (size_t) n;
   c->hmesh_cur = k;
   c->slot_pos.swap(pos);
   c->hw_slots = std::max(c->hw_slots, hw);
   mamr::batched_mesh_changed(c->batched);
   return MAMR_OK;
}

// ref/comm.c:162-203 turned into per-direction task lists for the current
// mesh: the same faces, in the same pairing, that the reference's on-rank
// loop visits (set_mesh has checked the mesh).
static int build_tasks(mamr_ctx *c)
{
   const mamr_ctx::MeshView &blocks = c->mesh;
   const std::vector<int32_t> &pos = c->slot_pos;
   const int32_t n = (int32_t) blocks.size();
   std::vector<SameTask> same[3];
   std::vector<DiffTask> diff[3];
   std::vector<BcTask> bc[3];
   for (int32_t in = 0; in < n; in++) {
      const mamr_block &bp = blocks[in];
      const int s = bp.slot;
      for (int l = 0; l < 6; l++) {
         const int dir = l / 2;
         if (bp.nei_level[l] == bp.level) {
            int m = bp.nei[l][0][0];
            if (m > s) {
               // l even: the neighbour is on the low side
               same[dir].push_back(l % 2 == 0 ? SameTask{m, s}
                                              : SameTask{s, m});
            }
         } else if (bp.nei_level[l] == bp.level + 1) {
            for (int i = 0; i < 2; i++)
               for (int j = 0; j < 2; j++) {
                  int m = bp.nei[l][i][j];
                  if (m > s)
                     diff[dir].push_back(DiffTask{s, m, l, i, j});
               }
         } else if (bp.nei_level[l] == bp.level - 1) {
            int m = bp.nei[l][0][0];
            if (m > s) {
               const mamr_block &mb = blocks[pos[m]];
               int k = dir * 2 + 1 - l % 2;
               for (int i = 0; i < 2; i++)
                  for (int j = 0; j < 2; j++)
                     if (mb.nei[k][i][j] == s)
                        diff[dir].push_back(DiffTask{m, s, k, i, j});
            }
         } else if (bp.nei_level[l] == -2) {
            bc[dir].push_back(BcTask{s, l});
         }
      }
   }
   // per direction: same | diff | bc
   for (int d = 0; d < 3; d++) {
      size_t b_same = same[d].size() * sizeof(SameTask);
      size_t b_diff = diff[d].size() * sizeof(DiffTask);
      size_t b_bc = bc[d].size() * sizeof(BcTask);
      size_t o_diff = (b_same + 15) & ~(size_t) 15;
      size_t o_bc = (o_diff + b_diff + 15) & ~(size_t) 15;
      std::vector<unsigned char> blob(o_bc + b_bc + 16);
      memcpy(blob.data(), same[d].data(), b_same);
      memcpy(blob.data() + o_diff, diff[d].data(), b_diff);
      memcpy(blob.data() + o_bc, bc[d].data(), b_bc);
      CUDA_TRY(c->d_tasks[d].ensure(blob.size()));
      CUDA_TRY(cudaMemcpyAsync(c->d_tasks[d].p, blob.data(), blob.size(),
                               cudaMemcpyHostToDevice, c->stream));
      unsigned char *base = (unsigned char *) c->d_tasks[d].p;
      c->tasks[d].same = (const SameTask *) base;
      c->tasks[d].n_same = (int) same[d].size();
      c->tasks[d].diff = (const DiffTask *) (base + o_diff);
      c->tasks[d].n_diff = (int) diff[d].size();
      c->tasks[d].bc = (const BcTask *) (base + o_bc);
      c->tasks[d].n_bc = (int) bc[d].size();
   }
   // the blobs are pageable host memory: let the copies take them before
   // they go
   CUDA_TRY(cudaStreamSynchronize(c->stream));
   c->tasks_dirty = false;
   return MAMR_OK;
}

static int comm_impl(mamr_ctx *c, int32_t start, int32_t num, int32_t stage)
{
   if (c->tasks_dirty) {
      const int r = build_tasks(c);
      if (r)
         return r;
   }
   // the cache serves the z exchange when it holds every variable of it
   bool zc = c->d_zc.p != nullptr && num > 0;
   for (int v = start; zc && v < start + num; v++)
      zc = c->zc_ok[v] != 0;
   for (int o = 0; o < 3; o++) {
      int dir = c->cfg.permute ? kPerm[((stage % 6) + 6) % 6][o] : o;
      if (c->fp32)
         LAUNCH_TRY(c, launch_comm_dir((float *) c->pool, c->g, dir,
                                       c->cfg.stencil, c->cfg.code,
                                       c->tasks[dir], start, num,
                                       zc ? (const float *) c->d_zc.p
                                          : nullptr,
                                       c->stream));
      else
         LAUNCH_TRY(c, launch_comm_dir((double *) c->pool, c->g, dir,
                                       c->cfg.stencil, c->cfg.code,
                                       c->tasks[dir], start, num,
                                       zc ? (const double *) c->d_zc.p
                                          : nullptr,
                                       c->stream));
   }
   return MAMR_OK;
}

extern "C" int mamr_comm(mamr_ctx *c, int32_t start, int32_t num,
                         int32_t stage)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (start < 0 || num < 0 || start + num > c->cfg.num_vars)
      return fail(MAMR_EINVAL, "variable range [%d, %d) out of bounds",
                  start, start + num);
   c->gen++;
   return comm_impl(c, start, num, stage);
}

static int stencil_impl(mamr_ctx *c, int32_t var, int32_t calc_stage,
                        bool per_block = false)
{
   const int n = (int) c->mesh.size();
   c->zface_live = -1;
   if (c->cfg.stencil == 0) {
      // stencil_driver (ref/stencil.c:43-74): var 0 and var >= 4*mat take
      // the 7-point stencil, the others the variable-work kernels
      const int mat = c->cfg.num_vars / 4;
      if (var != 0 && var < 4 * mat) {
         if (!c->work_set)
            return fail(MAMR_EINVAL, "stencil 0 needs mamr_set_work_params "
                        "before the first stencil");
         CUDA_TRY(c->d_work.ensure(sizeof(double) * std::max(1, n) *
                                   c->cfg.nx * c->cfg.ny * c->cfg.nz));
         if (!c->zc_ok.empty())
            c->zc_ok[var] = 0;
         LAUNCH_TRY(c, launch_work_stencil(
                          (double *) c->pool, c->g,
                          (const int32_t *) c->d_slots.p, n, var, calc_stage,
                          c->work, (double *) c->d_work.p, c->stream));
         return MAMR_OK;
      }
      double *zc = (double *) zcache_for_stencil(c);
      LAUNCH_TRY(c, launch_stencil((double *) c->pool, c->g, 7,
                                   (const int32_t *) c->d_slots.p, n, var, zc,
                                   c->stream));
      if (zc)
         c->zc_ok[var] = 1;
      return MAMR_OK;
   }
   void *zc = zcache_for_stencil(c);
   if (per_block) {
      for (int b = 0; b < n; b++) {
         const int32_t *one = (const int32_t *) c->d_slots.p + b;
         if (c->fp32)
            LAUNCH_TRY(c, launch_stencil((float *) c->pool, c->g,
                                         c->cfg.stencil, one, 1, var,
                                         (float *) zc, c->stream));
         else
            LAUNCH_TRY(c, launch_stencil((double *) c->pool, c->g,
                                         c->cfg.stencil, one, 1, var,
                                         (double *) zc, c->stream));
      }
   } else if (c->fp32) {
      LAUNCH_TRY(c, launch_stencil((float *) c->pool, c->g, c->cfg.stencil,
                                   (const int32_t *) c->d_slots.p, n, var,
                                   (float *) zc, c->stream));
   } else {
      LAUNCH_TRY(c, launch_stencil((double *) c->pool, c->g, c->cfg.stencil,
                                   (const int32_t *) c->d_slots.p, n, var,
                                   (double *) zc, c->stream));
   }
   if (zc)
      c->zc_ok[var] = 1;
   return MAMR_OK;
}

extern "C" int mamr_stencil(mamr_ctx *c, int32_t var, int32_t calc_stage)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (var < 0 || var >= c->cfg.num_vars)
      return fail(MAMR_EINVAL, "variable %d out of range", var);
   if (calc_stage < 0)
      return fail(MAMR_EINVAL, "negative calc_stage");
   c->gen++;
   return stencil_impl(c, var, calc_stage);
}

extern "C" int mamr_set_work_params(mamr_ctx *c, double a1, const double *a0,
                                    int32_t n_a0)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (c->cfg.stencil != 0)
      return fail(MAMR_EINVAL, "work parameters belong to stencil 0");
   if (!a0 || n_a0 != c->cfg.num_vars / 4)
      return fail(MAMR_EINVAL, "a0 must hold num_vars/4 = %d values",
                  c->cfg.num_vars / 4);
   c->work.mat = n_a0;
   c->work.a1 = a1;
   for (int q = 0; q < n_a0; q++)
      c->work.a0[q] = a0[q];
   c->work_set = true;
   return MAMR_OK;
}

// An FP32 checksum slot as a double: a 128-bit fixed-point accumulator
// (units of 2^-52) converted with one correct rounding, or -- under the
// fallback mark -- the compensated FP64 sum the fallback stored.
static double fixed_to_double(unsigned long long lo, unsigned long long hi)
{
   if (hi == kChecksumFallbackMark) {
      double d;
      memcpy(&d, &lo, sizeof(d));
      return d;
   }
   __int128 v = (__int128) (((unsigned __int128) hi << 64) |
                            (unsigned __int128) lo);
   return (double) v * 0x1p-52;
}

// Queues the checksum of var; FP64 into *d_out, FP32 into acc[2].
static int checksum_queue(mamr_ctx *c, int32_t var, double *d_out,
                          unsigned long long *acc)
{
   const int n = (int) c->mesh.size();
   if (c->fp32) {
      CUDA_TRY(c->d_csflags.ensure(3 * sizeof(unsigned)));
      unsigned *flags = (unsigned *) c->d_csflags.p;
      CUDA_TRY(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long),
                               c->stream));
      CUDA_TRY(cudaMemsetAsync(flags, 0, 3 * sizeof(unsigned), c->stream));
      LAUNCH_TRY(c, launch_checksum_fp32((const float *) c->pool, c->g,
                                         (const int32_t *) c->d_slots.p, n,
                                         var, acc, flags, c->stream));
      LAUNCH_TRY(c, launch_fp32_checksum_fallback(
                       (const float *) c->pool, c->g,
                       (const int32_t *) c->d_slots.p, n, var, 1, flags,
                       (double *) c->d_partials.p, acc, c->stream));
   } else {
      LAUNCH_TRY(c, launch_checksum_fp64((const double *) c->pool, c->g,
                                         (const int32_t *) c->d_slots.p, n,
                                         var, (double *) c->d_partials.p,
                                         d_out, c->stream));
   }
   return MAMR_OK;
}

extern "C" int mamr_check_sum(mamr_ctx *c, int32_t var, double *sum)
{
   if (!c || !sum)
      return fail(MAMR_EINVAL, "null argument");
   if (var < 0 || var >= c->cfg.num_vars)
      return fail(MAMR_EINVAL, "variable %d out of range", var);
   int r;
   if (!c->fp32) {
      // the driver asks for every variable in turn after a stage
      // (ref/driver.c:90-103): the first call sums them all at once, the
      // others read the result while the pool is unchanged
      if (c->cs_gen != c->gen) {
         const int V = c->cfg.num_vars;
         CUDA_TRY(c->d_cs.ensure(sizeof(double) * V));
         LAUNCH_TRY(c, launch_checksum_fp64_all(
                          (const double *) c->pool, c->g,
                          (const int32_t *) c->d_slots.p,
                          (int) c->mesh.size(), (double *) c->d_partials.p,
                          (double *) c->d_cs.p, c->stream));
         c->cs_host.resize(V);
         CUDA_TRY(cudaMemcpyAsync(c->cs_host.data(), c->d_cs.p,
                                  sizeof(double) * V, cudaMemcpyDeviceToHost,
                                  c->stream));
         if ((r = check_error_word(c)))
            return r;
         c->cs_gen = c->gen;
      }
      *sum = c->cs_host[var];
      return MAMR_OK;
   }
   r = checksum_queue(c, var, c->d_sum, c->d_acc);
   if (r)
      return r;
   if (c->fp32) {
      unsigned long long *h = (unsigned long long *) c->h_pinned;
      CUDA_TRY(cudaMemcpyAsync(h, c->d_acc, 2 * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, c->stream));
      if ((r = check_error_word(c)))
         return r;
      *sum = fixed_to_double(h[0], h[1]);
   } else {
      double *h = (double *) c->h_pinned;
      CUDA_TRY(cudaMemcpyAsync(h, c->d_sum, sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
      if ((r = check_error_word(c)))
         return r;
      *sum = *h;
   }
   return MAMR_OK;
}

template <int NR, int NW, typename Job, typename Reads, typename Writes,
          typename Launch>
static int run_segments(mamr_ctx *c, const Job *jobs_in, int32_t n,
                        Reads reads, Writes writes, Launch launch)
{
   const size_t elem = c->fp32 ? sizeof(float) : sizeof(double);
   const size_t block_bytes = (size_t) c->cfg.num_vars * c->g.bv * elem;
   std::vector<Job> jobs;
   std::vector<int32_t> staged;
   std::vector<Segment> segs;
   size_t max_stage = std::max<size_t>(8, (size_t(1) << 30) / block_bytes);
   for (;;) {
      jobs.assign(jobs_in, jobs_in + n);
      plan_segments<NR, NW>(jobs, c->cfg.max_blocks, max_stage, reads,
                            writes, staged, segs);
      size_t most = 0;
      for (const Segment &sg : segs)
         most = std::max(most, sg.stage_end - sg.stage_begin);
      cudaError_t e = c->d_xfer.ensure(std::max<size_t>(1, most) *
                                       block_bytes);
      if (e == cudaSuccess)
         break;
      cudaGetLastError();
      if (max_stage == 8)
         return fail(MAMR_ENOMEM, "no device memory for %zu staged blocks",
                     most);
      max_stage = 8;
   }
   CUDA_TRY(c->d_jobs.ensure(sizeof(Job) * jobs.size()));
   CUDA_TRY(c->d_xfer_slots.ensure(sizeof(int32_t) *
                                   std::max<size_t>(1, staged.size())));
   // the job list and the staged slots through the pinned ring: queued,
   // the caller's arrays free on return
   {
      const size_t bj = sizeof(Job) * (size_t) n;
      const size_t bs = sizeof(int32_t) * staged.size();
      const size_t os = (bj + 15) & ~(size_t) 15;
      int slot = 0;
      cudaError_t e;
      char *h = (char *) host_stage_take(c, os + bs + 16, &slot, &e);
      if (!h)
         return fail(MAMR_ECUDA, "host staging: %s", cudaGetErrorString(e));
      memcpy(h, jobs.data(), bj);
      if (bs)
         memcpy(h + os, staged.data(), bs);
      CUDA_TRY(cudaMemcpyAsync(c->d_jobs.p, h, bj, cudaMemcpyHostToDevice,
                               c->stream));
      if (bs)
         CUDA_TRY(cudaMemcpyAsync(c->d_xfer_slots.p, h + os, bs,
                                  cudaMemcpyHostToDevice, c->stream));
      CUDA_TRY(host_stage_queued(c, slot));
   }
   for (const Segment &sg : segs) {
      const int32_t *sl = (const int32_t *) c->d_xfer_slots.p + sg.stage_begin;
      const int ns = (int) (sg.stage_end - sg.stage_begin);
      if (c->fp32)
         LAUNCH_TRY(c, launch_stage_blocks((float *) c->d_xfer.p,
                                           (const float *) c->pool, c->g, sl,
                                           ns, c->stream));
      else
         LAUNCH_TRY(c, launch_stage_blocks((double *) c->d_xfer.p,
                                           (const double *) c->pool, c->g, sl,
                                           ns, c->stream));
      const Job *dj = (const Job *) c->d_jobs.p + sg.begin;
      LAUNCH_TRY(c, launch(dj, (int) (sg.end - sg.begin)));
   }
   return MAMR_OK;
}

extern "C" int mamr_split(mamr_ctx *c, const mamr_split_job *jobs, int32_t n)
{
   if (!c || n < 0 || (n && !jobs))
      return fail(MAMR_EINVAL, "bad split arguments");
   c->gen++;
   zcache_drop(c);
   for (int32_t t = 0; t < n; t++) {
      if (!slot_ok(c, jobs[t].parent))
         return fail(MAMR_EINVAL, "split parent slot %d out of range",
                     jobs[t].parent);
      for (int o = 0; o < 8; o++) {
         if (!slot_ok(c, jobs[t].child[o]))
            return fail(MAMR_EINVAL, "split child slot %d out of range",
                        jobs[t].child[o]);
         c->hw_slots = std::max(c->hw_slots, jobs[t].child[o] + 1);
      }
   }
   if (n == 0)
      return MAMR_OK;
   void *zf = zface_live_array(c);
   if (zf)
      for (int32_t t = 0; t < n; t++) {
         c->zface_ok[jobs[t].parent] = 0;
         for (int o = 0; o < 8; o++)
            c->zface_ok[jobs[t].child[o]] = 1;
      }
   return run_segments<1, 8>(
      c, jobs, n,
      [](mamr_split_job &j) { return std::array<int32_t *, 1>{&j.parent}; },
      [](mamr_split_job &j) {
         std::array<int32_t *, 8> w;
         for (int o = 0; o < 8; o++)
            w[o] = &j.child[o];
         return w;
      },
      [&](const mamr_split_job *dj, int m) {
         return c->fp32
                   ? launch_split((float *) c->pool,
                                  (const float *) c->d_xfer.p, c->g, dj, m,
                                  (float *) zf, c->stream)
                   : launch_split((double *) c->pool,
                                  (const double *) c->d_xfer.p, c->g, dj, m,
                                  (double *) zf, c->stream);
      });
}

extern "C" int mamr_consolidate(mamr_ctx *c, const mamr_consolidate_job *jobs,
                                int32_t n)
{
   if (!c || n < 0 || (n && !jobs))
      return fail(MAMR_EINVAL, "bad consolidate arguments");
   c->gen++;
   zcache_drop(c);
   for (int32_t t = 0; t < n; t++) {
      if (!slot_ok(c, jobs[t].target))
         return fail(MAMR_EINVAL, "consolidate target slot %d out of range",
                     jobs[t].target);
      c->hw_slots = std::max(c->hw_slots, jobs[t].target + 1);
      for (int o = 0; o < 8; o++)
         if (!slot_ok(c, jobs[t].child[o]))
            return fail(MAMR_EINVAL, "consolidate child slot %d out of range",
                        jobs[t].child[o]);
   }
   if (n == 0)
      return MAMR_OK;
   void *zf = zface_live_array(c);
   if (zf)
      for (int32_t t = 0; t < n; t++) {
         for (int o = 0; o < 8; o++)
            c->zface_ok[jobs[t].child[o]] = 0;
         c->zface_ok[jobs[t].target] = 1;
      }
   return run_segments<8, 1>(
      c, jobs, n,
      [](mamr_consolidate_job &j) {
         std::array<int32_t *, 8> r;
         for (int o = 0; o < 8; o++)
            r[o] = &j.child[o];
         return r;
      },
      [](mamr_consolidate_job &j) {
         return std::array<int32_t *, 1>{&j.target};
      },
      [&](const mamr_consolidate_job *dj, int m) {
         return c->fp32
                   ? launch_consolidate((float *) c->pool,
                                        (const float *) c->d_xfer.p, c->g, dj,
                                        m, (float *) zf, c->stream)
                   : launch_consolidate((double *) c->pool,
                                        (const double *) c->d_xfer.p, c->g,
                                        dj, m, (double *) zf, c->stream);
      });
}

// Plain stage loop: the driver's call sequence queued without host syncs;
// checksums land in a device array and come back once at the end.
static int run_plain(mamr_ctx *c, int32_t num_ts, int32_t spt, int32_t freq,
                     int32_t first_stage, bool per_block, double *sums,
                     int32_t *n_sums)
{
   c->zface_live = -1;
   const int V = c->cfg.num_vars;
   int per_ts = 0;
   if (freq)
      for (int st = 0; st < spt; st++)
         per_ts += !(st % freq);
   const size_t n_cs = (size_t) per_ts * num_ts;
   const size_t slot_bytes = c->fp32 ? 2 * sizeof(unsigned long long)
                                     : sizeof(double);
   CUDA_TRY(c->d_sums.ensure(std::max<size_t>(1, n_cs * V) * slot_bytes));
   if (c->fp32) {
      const size_t fb = std::max<size_t>(1, n_cs) * (2 + V) * sizeof(unsigned);
      CUDA_TRY(c->d_csflags.ensure(fb));
      CUDA_TRY(cudaMemsetAsync(c->d_csflags.p, 0, fb, c->stream));
   }
   int cnt = 0, gstage = first_stage, r;
   for (int ts = 0; ts < num_ts; ts++)
      for (int st = 0; st < spt; st++, gstage++) {
         const bool do_cs = freq && !(st % freq);
         if ((r = comm_impl(c, 0, V, gstage)))
            return r;
         for (int var = 0; var < V; var++)
            if ((r = stencil_impl(c, var, gstage, per_block)))
               return r;
         // every variable's checksum in one launch (a variable's stencil
         // writes only that variable, so the sums are those the driver's
         // per-variable calls return)
         if (do_cs && c->fp32) {
            unsigned long long *acc =
               (unsigned long long *) c->d_sums.p + 2 * (size_t) cnt * V;
            CUDA_TRY(cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long) *
                                                V,
                                     c->stream));
            unsigned *flags = (unsigned *) c->d_csflags.p +
                              (size_t) cnt * (2 + V);
            LAUNCH_TRY(c, launch_checksum_fp32_all(
                             (const float *) c->pool, c->g,
                             (const int32_t *) c->d_slots.p,
                             (int) c->mesh.size(), acc, flags, c->stream));
            LAUNCH_TRY(c, launch_fp32_checksum_fallback(
                             (const float *) c->pool, c->g,
                             (const int32_t *) c->d_slots.p,
                             (int) c->mesh.size(), 0, V, flags,
                             (double *) c->d_partials.p, acc, c->stream));
         }
         if (do_cs && !c->fp32)
            LAUNCH_TRY(c, launch_checksum_fp64_all(
                             (const double *) c->pool, c->g,
                             (const int32_t *) c->d_slots.p,
                             (int) c->mesh.size(), (double *) c->d_partials.p,
                             (double *) c->d_sums.p + (size_t) cnt * V,
                             c->stream));
         if (do_cs)
            cnt++;
      }
   if ((r = mamr_sync(c)))
      return r;
   if (sums && cnt) {
      if (c->fp32) {
         std::vector<unsigned long long> h((size_t) cnt * V * 2);
         CUDA_TRY(cudaMemcpy(h.data(), c->d_sums.p, h.size() * 8,
                             cudaMemcpyDeviceToHost));
         for (size_t q = 0; q < (size_t) cnt * V; q++)
            sums[q] = fixed_to_double(h[2 * q], h[2 * q + 1]);
      } else {
         CUDA_TRY(cudaMemcpy(sums, c->d_sums.p, sizeof(double) * cnt * V,
                             cudaMemcpyDeviceToHost));
      }
   }
   if (n_sums)
      *n_sums = cnt;
   return MAMR_OK;
}


// Per-block descriptors for the batched stage kernel, from the mesh.
static int build_items_host(mamr_ctx *c)
{
   BatchedState *B = c->batched;
   const int n = (int) c->mesh.size();
   // built straight into pinned memory (reused across meshes), so that the
   // upload runs at full copy speed
   if (B->h_cap < (size_t) std::max(1, n)) {
      if (B->h_items)
         cudaFreeHost(B->h_items);
      B->h_items = nullptr;
      B->h_cap = 0;
      const size_t want = (size_t) std::max(1, n) * 5 / 4 + 64;
      CUDA_TRY(cudaMallocHost((void **) &B->h_items, sizeof(BItem) * want));
      B->h_cap = want;
   }
   BItem *items = B->h_items;
   bool single = true;
   const int lev0 = n ? c->mesh[0].level : 0;
   for (int q = 0; q < n; q++)
      single = single && c->mesh[q].level == lev0;
   for (int q = 0; q < n; q++) {
      const mamr_block &bp = c->mesh[q];
      BItem &it = items[q];
      memset(&it, 0, sizeof(it));
      it.slot = bp.slot;
      for (int l = 0; l < 6; l++) {
         BFace &f = it.f[l];
         const int nl = bp.nei_level[l];
         if (nl == -2) {
            f.type = FACE_BC;
            it.bmask |= 1 << l;
         } else if (nl == bp.level) {
            f.type = FACE_SAME;
            f.nb[0] = bp.nei[l][0][0];
         } else if (nl == bp.level + 1) {
            f.type = FACE_FINE;
            for (int iq = 0; iq < 2; iq++)
               for (int jq = 0; jq < 2; jq++)
                  f.nb[iq * 2 + jq] = bp.nei[l][iq][jq];
         } else {
            f.type = FACE_COARSE;
            const int m = bp.nei[l][0][0];
            const int pm = c->slot_pos[m];
            if (pm < 0)
               return fail(MAMR_EMESH, "neighbour slot %d not active", m);
            bool found = false;
            for (int iq = 0; iq < 2 && !found; iq++)
               for (int jq = 0; jq < 2 && !found; jq++)
                  if (c->mesh[pm].nei[l ^ 1][iq][jq] == bp.slot) {
                     f.nb[0] = m;
                     f.iq = iq;
                     f.jq = jq;
                     found = true;
                  }
            if (!found)
               return fail(MAMR_EMESH, "slot %d is not a child face of its "
                           "coarser neighbour %d", bp.slot, m);
         }
      }
      set_jump_bits(it);
      // neighbours across edges and corners, for single-level meshes only
      // (27-point edge/corner ghosts and the pencil kernel's in-plane
      // neighbours; neither applies to a multi-level mesh): hop x, then y,
      // then z
      if (!single)
         continue;
      for (int dz = -1; dz <= 1; dz++)
         for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
               int cur = bp.slot;
               const int d[3] = {dx, dy, dz};
               for (int ax = 0; ax < 3 && cur >= 0; ax++) {
                  if (!d[ax])
                     continue;
                  const mamr_block &cb = c->mesh[c->slot_pos[cur]];
                  const int l = 2 * ax + (d[ax] > 0);
                  cur = (cb.nei_level[l] == cb.level) ? cb.nei[l][0][0] : -1;
                  if (cur >= 0 && c->slot_pos[cur] < 0)
                     cur = -1;
               }
               it.nb27[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)] =
                  cur >= 0 ? cur : bp.slot;
            }
   }
   // Pencils: chains of blocks along z from a lower z boundary to an upper
   // one, for single-level meshes of 16^3 blocks; every block must lie on
   // exactly one chain.
   std::vector<TileDesc> chain;
   std::vector<int2> pencils;
   B->n_pencils = 0;
   if (single && n > 0 && c->g.nx == 16 && c->g.ny == 16 && c->g.nz == 16) {
      std::vector<char> seen(n, 0);
      bool ok = true;
      for (int q = 0; q < n && ok; q++) {
         if (!(items[q].bmask & (1 << 4)))
            continue;
         int2 pc;
         pc.x = (int) chain.size();
         int cur = q;
         while (ok) {
            if (seen[cur]) { ok = false; break; }
            seen[cur] = 1;
            TileDesc td;
            td.slot = items[cur].slot;
            td.bmask = items[cur].bmask;
            for (int d = 0; d < 9; d++)
               td.nb9[d] = items[cur].nb27[9 + d];
            chain.push_back(td);
            if (items[cur].bmask & (1 << 5))
               break;
            const int up = items[cur].f[5].nb[0];
            cur = c->slot_pos[up];
            if (cur < 0)
               ok = false;
         }
         pc.y = (int) chain.size() - pc.x;
         if (pc.y > PENCIL_MAX)
            ok = false;
         pencils.push_back(pc);
      }
      for (int q = 0; q < n && ok; q++)
         ok = seen[q] != 0;
      if (ok) {
         CUDA_TRY(B->chain.ensure(sizeof(TileDesc) * chain.size()));
         CUDA_TRY(B->pencils.ensure(sizeof(int2) * pencils.size()));
         CUDA_TRY(cudaMemcpyAsync(B->chain.p, chain.data(),
                                  sizeof(TileDesc) * chain.size(),
                                  cudaMemcpyHostToDevice, c->stream));
         CUDA_TRY(cudaMemcpyAsync(B->pencils.p, pencils.data(),
                                  sizeof(int2) * pencils.size(),
                                  cudaMemcpyHostToDevice, c->stream));
         B->n_pencils = (int) pencils.size();
      }
   }
   const size_t n_items = (size_t) std::max(1, n);
   CUDA_TRY(B->items.ensure(sizeof(BItem) * n_items));
   CUDA_TRY(cudaMemcpyAsync(B->items.p, items, sizeof(BItem) * n_items,
                            cudaMemcpyHostToDevice, c->stream));
   CUDA_TRY(cudaStreamSynchronize(c->stream));
   B->n = n;
   B->single_level = single;
   B->valid = true;
   return MAMR_OK;
}

// The batched path's descriptors for the current mesh.  Meshes the pencil
// kernel takes (one level, 16^3 blocks) need the host-side z chains and
// are built on the host; every other mesh on the device, one thread per
// block, from the copy mamr_set_mesh uploaded (after a refinement of the
// 8^3 stress mesh, 24k blocks: about 1.6 ms on the host against tens of
// microseconds).  A mesh the device build rejects is built again on the
// host, which names what is wrong with it.
static int build_items_only(mamr_ctx *c);

static int build_items(mamr_ctx *c)
{
   BatchedState *B = c->batched;
   B->has_recipes = false;
   int r = build_items_only(c);
   if (r != MAMR_OK || B->single_level || c->cfg.stencil != 27)
      return r;
   // multi-level 27-point: the edge and corner recipes, built on the
   // device from the mesh copy (one thread per block and recipe)
   const int n = B->n;
   CUDA_TRY(B->recipes.ensure(sizeof(GhostRecipe) * kGhostRecipes *
                              (size_t) std::max(1, n)));
   CUDA_TRY(B->keep.ensure(sizeof(int) * (size_t) std::max(1, n)));
   CUDA_TRY(B->bad.ensure(sizeof(int)));
   CUDA_TRY(cudaMemsetAsync(B->bad.p, 0x7f, sizeof(int), c->stream));
   if (launch_build_recipes((const mamr_block *) c->d_mesh.p, n,
                            (const int32_t *) c->d_slot_pos.p, c->g,
                            (GhostRecipe *) B->recipes.p, (int *) B->keep.p,
                            (int *) B->bad.p, c->stream) < 0)
      return fail(MAMR_ECUDA, "recipe build: %s",
                  cudaGetErrorString(cudaGetLastError()));
   c->launches++;
   int bad = 0;
   CUDA_TRY(cudaMemcpyAsync(&bad, B->bad.p, sizeof(int),
                            cudaMemcpyDeviceToHost, c->stream));
   CUDA_TRY(cudaStreamSynchronize(c->stream));
   if (bad != 0x7f7f7f7f) {
      B->valid = false;
      return fail(MAMR_EMESH, "misconnected block (slot %d): an edge or "
                  "corner ghost crosses a face whose neighbour does not "
                  "list it", c->mesh[bad].slot);
   }
   B->has_recipes = true;
   return MAMR_OK;
}

static int build_items_only(mamr_ctx *c)
{
   BatchedState *B = c->batched;
   const int n = (int) c->mesh.size();
   bool single = true;
   for (int q = 0; q < n; q++)
      single = single && c->mesh[q].level == c->mesh[0].level;
   if (single && n > 0 && c->g.nx == 16 && c->g.ny == 16 && c->g.nz == 16)
      return build_items_host(c);
   CUDA_TRY(B->items.ensure(sizeof(BItem) * (size_t) std::max(1, n)));
   CUDA_TRY(B->bad.ensure(sizeof(int)));
   CUDA_TRY(cudaMemsetAsync(B->bad.p, 0x7f, sizeof(int), c->stream));
   if (launch_build_items((const mamr_block *) c->d_mesh.p, n,
                          (const int32_t *) c->d_slot_pos.p, single ? 1 : 0,
                          (BItem *) B->items.p, (int *) B->bad.p,
                          c->stream) < 0)
      return fail(MAMR_ECUDA, "descriptor build: %s",
                  cudaGetErrorString(cudaGetLastError()));
   int bad = 0;
   CUDA_TRY(cudaMemcpyAsync(&bad, B->bad.p, sizeof(int),
                            cudaMemcpyDeviceToHost, c->stream));
   CUDA_TRY(cudaStreamSynchronize(c->stream));
   if (bad != 0x7f7f7f7f)
      return build_items_host(c);
   B->n = n;
   B->single_level = single;
   B->n_pencils = 0;
   B->valid = true;
   return MAMR_OK;
}

// The stage loop of ref/driver.c:73-108 as one fused launch per stage.
// ---- launch-shape autotuner ----------------------------------------------
// Stage indices of the tuner's stages (a run's stages count from 0).
constexpr int kTunePrime = -2, kTuneTimed = -3;
// The first batched run for each (block shape, stencil, precision, kernel,
// work size, checksum frequency) times every candidate shape of the stage
// kernel -- one warm-up and three timed stages each, current pool into the
// spare pool, checksums as the run takes them, no ghost writes, z-face
// arrays as after a run's first stage -- and keeps the fastest for the
// process.
// MAMR_TUNE=off in the environment keeps the first (default) candidate.
namespace {
struct TuneKey {
   int nx, ny, nz, stencil, fp32, pencil, work_log2, n_cands, freq;
   bool operator<(const TuneKey &o) const
   {
      return std::tie(nx, ny, nz, stencil, fp32, pencil, work_log2, n_cands,
                      freq) <
             std::tie(o.nx, o.ny, o.nz, o.stencil, o.fp32, o.pencil,
                      o.work_log2, o.n_cands, o.freq);
   }
};
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune_best;

bool tuning_disabled()
{
   const char *e = getenv("MAMR_TUNE");
   return e && (!strcmp(e, "off") || !strcmp(e, "0"));
}
}  // namespace

template <typename Stage>
static int tune_choice(mamr_ctx *c, const std::vector<StageShape> &cands,
                       bool pencil, int nb, int freq, int scratch_cs,
                       Stage &stage, int &choice, bool *timed)
{
   choice = 0;
   *timed = false;
   if (cands.size() < 2 || tuning_disabled())
      return MAMR_OK;
   long long work = (long long) nb * c->cfg.num_vars;
   int lg = 0;
   while (work > 1) {
      work >>= 1;
      lg++;
   }
   const TuneKey key{c->g.nx, c->g.ny, c->g.nz, c->cfg.stencil,
                     c->fp32 ? 1 : 0, pencil ? 1 : 0, lg,
                     (int) cands.size(), std::min(freq, 8)};
   {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune_best.find(key);
      if (it != g_tune_best.end()) {
         choice = it->second;
         return MAMR_OK;
      }
   }
   *timed = true;      // its stages write over both z-face arrays
   cudaEvent_t e0 = nullptr, e1 = nullptr;
   CUDA_TRY(cudaEventCreate(&e0));
   if (cudaEventCreate(&e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      return fail(MAMR_ECUDA, "event creation failed");
   }
   float best = 0.f;
   int status = MAMR_OK;
   // the kernels with z-face arrays are timed as the stages after a run's
   // first run them, reading one array and writing the other: a priming
   // stage of the first such candidate fills the array they read
   for (size_t q = 0; q < cands.size(); q++)
      if (cands[q].kernel == 1 || cands[q].kernel == 2) {
         const int k = stage(c->pool, c->pool_alt, cands[q], 0, false, 0,
                             kTunePrime);
         if (k < 0) {
            status = fail(MAMR_ECUDA, "priming stage: %s",
                          cudaGetErrorString(cudaGetLastError()));
            break;
         }
         c->launches += k;
         break;
      }
   // the timed stages take checksums as the run's stages do (stage t of
   // the three when t % freq == 0), into the scratch checksum slot
   for (size_t q = 0; q < cands.size() && status == MAMR_OK; q++) {
      int k = stage(c->pool, c->pool_alt, cands[q], 0, false, scratch_cs,
                    kTuneTimed);
      bool ok = k >= 0;
      c->launches += ok ? k : 0;
      ok = ok && cudaEventRecord(e0, c->stream) == cudaSuccess;
      for (int rep = 0; rep < 3 && ok; rep++) {
         k = stage(c->pool, c->pool_alt, cands[q], 0, freq && !(rep % freq),
                   scratch_cs, kTuneTimed);
         ok = k >= 0;
         c->launches += ok ? k : 0;
      }
      ok = ok && cudaEventRecord(e1, c->stream) == cudaSuccess;
      ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.f;
      ok = ok && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      if (!ok) {
         status = fail(MAMR_ECUDA, "timing launch shape %zu: %s", q,
                       cudaGetErrorString(cudaGetLastError()));
         break;
      }
      if (q == 0 || ms < best) {
         best = ms;
         choice = (int) q;
      }
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   if (status == MAMR_OK) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune_best[key] = choice;
   }
   return status;
}

static int run_batched(mamr_ctx *c, int32_t num_ts, int32_t spt,
                       int32_t freq, bool graph, bool ghosts_out,
                       double *sums, int32_t *n_sums)
{
   int r;
   zcache_drop(c);
   if (!c->batched) {
      c->batched = new (std::nothrow) BatchedState();
      if (!c->batched)
         return fail(MAMR_ENOMEM, "host allocation");
   }
   BatchedState *B = c->batched;
   // the z-face array the previous run left live (if any), and none live
   // until this run completes
   const int live0 = c->zface_live;
   c->zface_live = -1;
   if (!B->valid && (r = build_items(c)))
      return r;
   if (c->cfg.stencil == 0)
      return fail(MAMR_EUNSUP, "the batched path runs stencils 7 and 27; "
                  "stencil 0 runs on the plain path");
   if (c->cfg.code != 0)
      return fail(MAMR_EUNSUP, "the batched path gathers code-0 ghosts; "
                  "code %d runs on the plain path", c->cfg.code);
   if (c->cfg.stencil == 27 && c->cfg.permute)
      return fail(MAMR_EUNSUP, "batched 27-point stencil with --permute: "
                  "with the phases reordered, edge and corner ghosts take "
                  "neighbours' ghost values of the previous stage, which "
                  "one fused launch per stage does not keep; the plain "
                  "path runs it");
   const int V = c->cfg.num_vars, nb = B->n;
   int per_ts = 0;
   if (freq)
      for (int st = 0; st < spt; st++)
         per_ts += !(st % freq);
   const size_t n_cs = (size_t) per_ts * num_ts;
   const size_t es = elem_size(c);
   if (!c->pool_alt)
      CUDA_TRY(pool_alloc(c, &c->pool_alt));
   CUDA_TRY(B->partials.ensure(sizeof(double) * std::max(1, nb) * V));
   // checksum slots: one per checksum stage, and a scratch slot (n_cs) for
   // the tuner's stages
   if (c->fp32) {
      CUDA_TRY(B->acc.ensure((n_cs + 1) * V * 16));
      CUDA_TRY(cudaMemsetAsync(B->acc.p, 0, (n_cs + 1) * V * 16, c->stream));
      const size_t fb = (n_cs + 1) * (2 + V) * sizeof(unsigned);
      CUDA_TRY(B->csflags.ensure(fb));
      CUDA_TRY(cudaMemsetAsync(B->csflags.p, 0, fb, c->stream));
   } else {
      CUDA_TRY(B->sums.ensure(sizeof(double) * (n_cs + 1) * V));
   }
   const bool pencil = B->n_pencils > 0;
   const int np = B->n_pencils;
   // stale edge/corner ghosts (multi-level 27-point) are read from the pool
   // the run starts from: no stage before the last writes ghosts anywhere
   const void *stale_pool = c->pool;
   const GhostRecipe *recipes =
      B->has_recipes ? (const GhostRecipe *) B->recipes.p : nullptr;
   const int *keep = B->has_recipes ? (const int *) B->keep.p : nullptr;
   // one stage: cur -> oth with launch shape sh; q = the stage's index in
   // the run, or a tuning stage (kTunePrime, kTuneTimed).  The
   // warp-per-block and tile kernels write the z-face array (zb + q) & 1
   // and read the one stage q - 1 wrote -- the first stage the array the
   // previous run left live when it holds every active block (first_in);
   // tuning stages write array 0 (priming) or read array 0 and write
   // array 1 (timed).
   int zb = 0, first_in = -1;
   auto stage = [&](const void *cur, void *oth, const StageShape &sh,
                    int last, bool do_cs, int cnt, int q) -> int {
      const bool zk = sh.kernel == 1 || sh.kernel == 2;
      int zin = -1, zout = -1;
      if (zk && q >= 0) {
         zout = (zb + q) & 1;
         zin = q > 0 ? (zb + q - 1) & 1 : first_in;
      } else if (zk && q == kTunePrime) {
         zout = 0;
      } else if (zk && q == kTuneTimed) {
         zin = 0;
         zout = 1;
      }
      void *zf_dst = zout >= 0 ? B->zf[zout].p : nullptr;
      const void *zf_src = zin >= 0 ? B->zf[zin].p : nullptr;
      unsigned long long *acc =
         c->fp32 ? (unsigned long long *) B->acc.p + (size_t) cnt * V * 2
                 : nullptr;
      double *sums_at =
         c->fp32 ? nullptr : (double *) B->sums.p + (size_t) cnt * V;
      double *part = c->fp32 ? nullptr : (double *) B->partials.p;
      // FP32 checksum stages: the stage kernel reports cells outside the
      // fixed-point window in the stage's miss word, and the fallback
      // (empty unless it was set) replaces those variables' sums
      unsigned *flags = c->fp32 && do_cs
                           ? (unsigned *) B->csflags.p + (size_t) cnt * (2 + V)
                           : c->d_err;
      auto fallback = [&](int k) -> int {
         if (k < 0 || !c->fp32 || !do_cs)
            return k;
         const int f = launch_fp32_checksum_fallback(
            (const float *) oth, c->g, (const int32_t *) c->d_slots.p, nb, 0,
            V, flags, (double *) B->partials.p, acc, c->stream);
         return f < 0 ? -1 : k + f;
      };
      const long long n_bv = (long long) c->cfg.max_blocks * V;
      if (pencil && c->fp32)
         return fallback(launch_pencil_stage(
            (const float *) cur, (float *) oth, c->g, c->cfg.stencil,
            (const BItem *) B->items.p, nb, (const TileDesc *) B->chain.p,
            (const int2 *) B->pencils.p, np, sh, last, do_cs, part, sums_at,
            acc, flags, c->d_err, n_bv, c->stream));
      if (pencil)
         return launch_pencil_stage((const double *) cur, (double *) oth,
                                    c->g, c->cfg.stencil,
                                    (const BItem *) B->items.p, nb,
                                    (const TileDesc *) B->chain.p,
                                    (const int2 *) B->pencils.p, np, sh, last,
                                    do_cs, part, sums_at, acc, c->d_err,
                                    c->d_err, n_bv, c->stream);
      if (c->fp32)
         return fallback(launch_batched_stage(
            (const float *) cur, (float *) oth, c->g, c->cfg.stencil,
            (const BItem *) B->items.p, recipes, keep,
            (const float *) stale_pool,
            nb, sh, last, do_cs, part, sums_at, acc, flags, c->d_err, n_bv,
            (const float *) zf_src, (float *) zf_dst, c->stream));
      return launch_batched_stage((const double *) cur, (double *) oth, c->g,
                                  c->cfg.stencil, (const BItem *) B->items.p,
                                  recipes, keep, (const double *) stale_pool,
                                  nb,
                                  sh, last, do_cs, part, sums_at, acc,
                                  c->d_err, c->d_err, n_bv,
                                  (const double *) zf_src,
                                  (double *) zf_dst, c->stream);
   };
   std::vector<StageShape> cands;
   if (pencil && c->fp32)
      pencil_candidates<float>(c->cfg.stencil, np * V, cands);
   else if (pencil)
      pencil_candidates<double>(c->cfg.stencil, np * V, cands);
   else if (c->fp32)
      batched_candidates<float>(c->g, c->cfg.stencil, nb, cands);
   else
      batched_candidates<double>(c->g, c->cfg.stencil, nb, cands);
   CUDA_TRY(cudaGetLastError());
   if (cands.empty())
      return fail(MAMR_EUNSUP, "no launch shape of the batched stage kernel "
                  "fits blocks of %d x %d x %d cells; the plain path runs "
                  "them", c->g.nx, c->g.ny, c->g.nz);
   // the warp-per-block and tile kernels' z-face arrays (written by each
   // stage, read by the next; the tuner times those kernels with them)
   for (const StageShape &cd : cands)
      if (cd.kernel == 1 || cd.kernel == 2) {
         const size_t zbytes = zface_elems(c->g, c->cfg.max_blocks) * es;
         CUDA_TRY(B->zf[0].ensure(zbytes));
         CUDA_TRY(B->zf[1].ensure(zbytes));
         break;
      }
   int choice = 0;
   bool tuned_now = false;
   if (c->tune_force >= 0) {
      choice = std::min<int>(c->tune_force, (int) cands.size() - 1);
   } else if ((r = tune_choice(c, cands, pencil, nb, freq, (int) n_cs, stage,
                               choice, &tuned_now))) {
      return r;
   }
   const StageShape sh = cands[choice];
   c->tune_last = choice;
   c->tune_n = (int) cands.size();
   c->tune_shape = sh;
   const bool zkern = sh.kernel == 1 || sh.kernel == 2;
   // the first stage reads the z-face array the previous run left, if no
   // tuning stage has written over it and it holds every active block
   if (zkern && live0 >= 0 && !tuned_now && B->zf[live0].p) {
      bool all = true;
      for (const mamr_block &b : c->mesh)
         all = all && c->zface_ok[b.slot];
      if (all) {
         first_in = live0;
         zb = 1 - live0;
      }
   }
   // A run of an odd number of stages ends in the spare pool: it must then
   // hold what no stage writes (stale ghosts, free slots) as the current
   // pool does, so it starts as a copy.  With an even number the run ends
   // in the current pool and no stage reads a spare-pool cell that an
   // earlier stage of the run did not write, so no copy is needed (the
   // tuner above wrote only interiors of the spare pool).
   const size_t used = (size_t) c->hw_slots * c->g.V * c->g.bv * es;
   if (used && (num_ts * spt) % 2 == 1)
      CUDA_TRY(cudaMemcpyAsync(c->pool_alt, c->pool, used,
                               cudaMemcpyDeviceToDevice, c->stream));

   cudaGraph_t g_graph = nullptr;
   if (graph)
      CUDA_TRY(cudaStreamBeginCapture(c->stream,
                                      cudaStreamCaptureModeThreadLocal));
   void *cur = c->pool, *oth = c->pool_alt;
   long long launches = 0;
   int cnt = 0, status = MAMR_OK;
   const int total = num_ts * spt;
   for (int ts = 0, q = 0; ts < num_ts && status == MAMR_OK; ts++)
      for (int st = 0; st < spt; st++, q++) {
         const bool do_cs = freq && !(st % freq);
         const int last = ghosts_out && q == total - 1;
         const int k = stage(cur, oth, sh, last, do_cs, cnt, q);
         if (k < 0) {
            status = fail(MAMR_ECUDA, "batched stage launch: %s",
                          cudaGetErrorString(cudaGetLastError()));
            break;
         }
         launches += k;
         if (do_cs)
            cnt++;
         std::swap(cur, oth);
      }
   if (graph) {
      cudaError_t e = cudaStreamEndCapture(c->stream, &g_graph);
      if (status != MAMR_OK) {
         if (g_graph)
            cudaGraphDestroy(g_graph);
         return status;
      }
      if (e != cudaSuccess)
         return fail(MAMR_ECUDA, "graph capture: %s", cudaGetErrorString(e));
      cudaGraphExec_t exec = nullptr;
      e = cudaGraphInstantiate(&exec, g_graph, 0);
      if (e == cudaSuccess)
         e = cudaGraphLaunch(exec, c->stream);
      if (exec)
         cudaGraphExecDestroy(exec);
      cudaGraphDestroy(g_graph);
      if (e != cudaSuccess)
         return fail(MAMR_ECUDA, "graph launch: %s", cudaGetErrorString(e));
   } else if (status != MAMR_OK) {
      return status;
   }
   c->launches += launches;
   if (cur != c->pool) {
      std::swap(c->pool, c->pool_alt);
   }
   if (zkern && total > 0 && B->zf[(zb + total - 1) & 1].p) {
      // the last stage wrote every active block's planes
      c->zface_live = (zb + total - 1) & 1;
      std::fill(c->zface_ok.begin(), c->zface_ok.end(), 0);
      for (const mamr_block &b : c->mesh)
         c->zface_ok[b.slot] = 1;
   }
   if ((r = mamr_sync(c)))
      return r;
   if (sums && cnt) {
      if (c->fp32) {
         std::vector<unsigned long long> h((size_t) cnt * V * 2);
         CUDA_TRY(cudaMemcpy(h.data(), B->acc.p, h.size() * 8,
                             cudaMemcpyDeviceToHost));
         for (size_t q = 0; q < (size_t) cnt * V; q++)
            sums[q] = fixed_to_double(h[2 * q], h[2 * q + 1]);
      } else {
         CUDA_TRY(cudaMemcpy(sums, B->sums.p, sizeof(double) * cnt * V,
                             cudaMemcpyDeviceToHost));
      }
   }
   if (n_sums)
      *n_sums = cnt;
   return MAMR_OK;
}

extern "C" int mamr_run_timesteps(mamr_ctx *c, int32_t num_ts,
                                  int32_t stages_per_ts,
                                  int32_t checksum_freq, int32_t first_stage,
                                  int32_t flags, double *sums,
                                  int32_t *n_sums)
{
   if (!c || num_ts < 0 || stages_per_ts < 1 || checksum_freq < 0)
      return fail(MAMR_EINVAL, "bad run arguments");
   c->gen++;
   if (flags & ~(MAMR_RUN_BATCHED | MAMR_RUN_GRAPH | MAMR_RUN_PER_BLOCK |
                 MAMR_RUN_NO_GHOSTS))
      return fail(MAMR_EINVAL, "unknown run flags 0x%x", flags);
   if ((flags & MAMR_RUN_NO_GHOSTS) &&
       (!(flags & MAMR_RUN_BATCHED) || c->cfg.stencil != 7))
      return fail(MAMR_EINVAL, "MAMR_RUN_NO_GHOSTS needs MAMR_RUN_BATCHED "
                  "and the 7-point stencil");
   if (!(flags & MAMR_RUN_BATCHED)) {
      if (flags & MAMR_RUN_GRAPH)
         return fail(MAMR_EINVAL, "MAMR_RUN_GRAPH needs MAMR_RUN_BATCHED");
      return run_plain(c, num_ts, stages_per_ts, checksum_freq, first_stage,
                       (flags & MAMR_RUN_PER_BLOCK) != 0, sums, n_sums);
   }
   if (flags & MAMR_RUN_PER_BLOCK)
      return fail(MAMR_EINVAL, "MAMR_RUN_PER_BLOCK applies to the plain path");
   return run_batched(c, num_ts, stages_per_ts, checksum_freq,
                      (flags & MAMR_RUN_GRAPH) != 0,
                      (flags & MAMR_RUN_NO_GHOSTS) == 0, sums, n_sums);
}

// mamr_mark_validate for long block lists: the per-block checks spread
// over kHostThreads threads, each slot's mark set by an atomic exchange (a
// slot listed twice finds its mark already set).  On any failure the
// serial check runs again on a cleared mark array, so that the message is
// the one it returns.
static const char *mark_validate(const mamr_mark_params *p,
                                 const mamr_object *objs, int32_t n_objs,
                                 const mamr_mark_block *mb, int32_t nb,
                                 const mamr_mark_parent *pa, int32_t np,
                                 int32_t cap, unsigned char *listed)
{
   if (nb < 4096 || !mb)
      return mamr_mark_validate(p, objs, n_objs, mb, nb, pa, np, cap, listed);
   // parameters and parents (nothing listed yet)
   int bad = mamr_mark_validate(p, objs, n_objs, mb, 0, pa, np, cap,
                                listed) != nullptr;
   if (!bad) {
#pragma omp parallel for num_threads(kHostThreads) schedule(static) \
   reduction(| : bad)
      for (int32_t i = 0; i < nb; i++) {
         const mamr_mark_block &b = mb[i];
         if (b.slot < 0 || b.slot >= cap || b.level < 0 ||
             b.level > p->num_refine || b.parent < -1 || b.parent >= np)
            bad = 1;
         else if (__atomic_exchange_n(&listed[b.slot], (unsigned char) 1,
                                      __ATOMIC_RELAXED))
            bad = 1;
      }
   }
   if (!bad) {
#pragma omp parallel for num_threads(kHostThreads) schedule(static) \
   reduction(| : bad)
      for (int32_t i = 0; i < nb; i++)
         for (int l = 0; l < 6; l++) {
            const int nl = mb[i].nei_level[l], n = mb[i].nei[l];
            if ((nl == mb[i].level || nl == mb[i].level - 1) &&
                (n < 0 || n >= cap || !listed[n]))
               bad = 1;
         }
   }
   if (!bad)
      return nullptr;
   std::memset(listed, 0, (size_t) cap + 1);
   return mamr_mark_validate(p, objs, n_objs, mb, nb, pa, np, cap, listed);
}

extern "C" int mamr_mark_refine(mamr_ctx *c, const mamr_mark_params *p,
                                const mamr_object *objs, int32_t n_objs,
                                const mamr_mark_block *mb, int32_t nb,
                                const mamr_mark_parent *pa, int32_t np,
                                int32_t *block_refine, int32_t *parent_refine)
{
   if (!c || (nb && !block_refine) || (np && !parent_refine))
      return fail(MAMR_EINVAL, "mark_refine: bad arguments");
   // callable from any host thread: the context's device
   int cur_dev = -1;
   if (cudaGetDevice(&cur_dev) == cudaSuccess && cur_dev != c->device)
      CUDA_TRY(cudaSetDevice(c->device));
   const int32_t cap = c->cfg.max_blocks;
   std::vector<unsigned char> listed((size_t) cap + 1, 0);
   if (const char *msg = mark_validate(p, objs, n_objs, mb, nb, pa, np, cap,
                                       listed.data()))
      return fail(MAMR_EINVAL, "%s", msg);
   // one device allocation: objects, blocks, parents, flags by slot,
   // parent flags, output, each 256-byte aligned
   auto up = [](size_t b) { return (b + 255) & ~(size_t) 255; };
   const size_t b_obj = up(sizeof(mamr_object) * n_objs),
                b_mb = up(sizeof(mamr_mark_block) * nb),
                b_pa = up(sizeof(mamr_mark_parent) * np),
                b_ref = up(sizeof(int32_t) * cap),
                b_pref = up(sizeof(int32_t) * np),
                b_out = up(sizeof(int32_t) * nb), b_flags = up(3 * sizeof(int));
   CUDA_TRY(c->d_mark.ensure(b_obj + b_mb + b_pa + b_ref + b_pref + b_out +
                             b_flags));
   char *base = (char *) c->d_mark.p;
   mamr_object *d_obj = (mamr_object *) base;
   mamr_mark_block *d_mb = (mamr_mark_block *) (base + b_obj);
   mamr_mark_parent *d_pa = (mamr_mark_parent *) (base + b_obj + b_mb);
   int32_t *d_ref = (int32_t *) (base + b_obj + b_mb + b_pa);
   int32_t *d_pref = (int32_t *) ((char *) d_ref + b_ref);
   int32_t *d_out = (int32_t *) ((char *) d_pref + b_pref);
   int *d_flags = (int *) ((char *) d_out + b_out);
   if (n_objs)
      CUDA_TRY(cudaMemcpyAsync(d_obj, objs, sizeof(mamr_object) * n_objs,
                               cudaMemcpyHostToDevice, c->stream));
   if (nb)
      CUDA_TRY(cudaMemcpyAsync(d_mb, mb, sizeof(mamr_mark_block) * nb,
                               cudaMemcpyHostToDevice, c->stream));
   if (np)
      CUDA_TRY(cudaMemcpyAsync(d_pa, pa, sizeof(mamr_mark_parent) * np,
                               cudaMemcpyHostToDevice, c->stream));
   const int k = launch_mark_refine(
      *p, make_int3(c->cfg.nx, c->cfg.ny, c->cfg.nz), d_obj, n_objs, d_mb,
      nb, d_pa, np, cap, d_ref, d_pref, d_out, d_flags, c->d_err, c->stream);
   if (k < 0)
      return fail(MAMR_ECUDA, "mark_refine launch: %s",
                  cudaGetErrorString(cudaGetLastError()));
   c->launches += k;
   std::vector<int32_t> hp((size_t) np);
   if (nb)
      CUDA_TRY(cudaMemcpyAsync(block_refine, d_out, sizeof(int32_t) * nb,
                               cudaMemcpyDeviceToHost, c->stream));
   if (np)
      CUDA_TRY(cudaMemcpyAsync(hp.data(), d_pref, sizeof(int32_t) * np,
                               cudaMemcpyDeviceToHost, c->stream));
   int r = check_error_word(c);        // synchronises the stream
   if (r)
      return r;
   for (int32_t q = 0; q < np; q++)
      if (pa[q].active)
         parent_refine[q] = hp[q];
   return MAMR_OK;
}

extern "C" int mamr_set_tuning(mamr_ctx *c, int32_t choice)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   c->tune_force = choice < 0 ? -1 : choice;
   return MAMR_OK;
}

extern "C" int mamr_get_tuning(const mamr_ctx *c, int32_t *choice,
                               int32_t *n_candidates, int32_t *shape)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (choice)
      *choice = c->tune_last;
   if (n_candidates)
      *n_candidates = c->tune_n;
   if (shape) {
      const StageShape &sh = c->tune_shape;
      const bool brick = sh.kernel == 1;
      shape[0] = sh.threads;
      // the warp-per-block kernel: variables per CTA = items x variables
      // per item, and i-planes 0 (-1: its tensor-copy form)
      shape[1] = brick ? sh.vpc * std::max(1, sh.planes) : sh.vpc;
      shape[2] = sh.rows;
      shape[3] = brick ? (sh.tma ? -1 : 0) : sh.planes;
      shape[4] = sh.grid;
   }
   return MAMR_OK;
}
