// binning.cu -- deterministic tile binning with a hand-written onesweep LSD
// radix sort.
//
// The reference (gs/src/include/aabb_culling.h:15-41, 192-260) emits one
// 64-bit key (tile_id << 32 | float bits of depth) per (Gaussian, tile of its
// AABB) through a global atomic counter, sorts all 64 bits with CUB, and
// derives start/end from the sorted tile ids (:70-103).  The same ordering is
// produced here with far less K-sized traffic:
//   1. sort the n Gaussians by depth bits (4 passes over n, not K, items);
//   2. exclusive scan of their key counts in that order (decoupled look-back)
//      and emission of (tile, Gaussian) pairs -- deterministic, no atomics;
//   3. stable sort of the K pairs by tile id: ceil(log2(tiles)/8) passes;
//   4. start/end from the tile boundaries.
// Equal (tile, depth) keys come out in Gaussian-index order, i.e. the
// reference's order after its non-deterministic ties are canonicalised.
//
// Onesweep pass (one launch per 8-bit digit): each CTA claims the next chunk
// of 4096 keys through an atomic ticket (so every chunk it waits on belongs
// to a CTA that is already running), ranks its keys stably per digit with
// warp match + per-warp counters, publishes its digit counts, looks back over
// the preceding chunks' counts for its global offsets, and scatters through
// shared memory so that the global writes are runs of consecutive addresses.
// Every wait on a predecessor is bounded; on expiry an error word is set and
// the host returns GSX_ERR_TIMEOUT.
#include <algorithm>

#include "gsx_internal.cuh"

namespace gsx {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // keys per chunk (8-bit digits)
// 9-bit digits (two passes for 17-18-bit tile ids, e.g. a batch of views
// with up to 2^18 tiles): 512 buckets, 12 keys per thread to stay within
// 48 KB of static shared memory
constexpr int kItems9 = 12;
constexpr int kTileMin = kThreads * kItems9;  // smallest chunk: sizes the look-back rows
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kEmitItems = 2;
constexpr int kEmitTile = kThreads * kEmitItems;
constexpr unsigned long long kFlag64Agg = 1ull << 62;
constexpr unsigned long long kFlag64Prefix = 2ull << 62;
constexpr unsigned long long kCount64Mask = (1ull << 62) - 1ull;

// error word bits
constexpr uint32_t kErrTimeout = 1u;
constexpr uint32_t kErrCount = 2u;
constexpr uint32_t kErrRange = 4u;  // rectangle outside the tile grid
constexpr uint32_t kErrIndex = 8u;  // corrupted depth order (after a timeout)
constexpr size_t kStatusBlockBytes = 16;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *reinterpret_cast<const volatile uint32_t *>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) {
  *reinterpret_cast<volatile uint32_t *>(p) = v;
}
__device__ __forceinline__ unsigned long long ld_volatile64(const unsigned long long *p) {
  return *reinterpret_cast<const volatile unsigned long long *>(p);
}
__device__ __forceinline__ void st_volatile64(unsigned long long *p, unsigned long long v) {
  *reinterpret_cast<volatile unsigned long long *>(p) = v;
}

// Exclusive scan of one value per thread over a 256-thread block.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *s_tmp, T *total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_tmp[w] = x;
  __syncthreads();
  T wsum = 0, all = 0;
#pragma unroll
  for (int k = 0; k < kWarps; ++k) {
    T c = s_tmp[k];
    if (k < w) wsum += c;
    all += c;
  }
  __syncthreads();
  if (total) *total = all;
  return x - v + wsum;
}

// The lanes of the warp whose (valid) digit equals this lane's.  BALLOT: one
// ballot per digit bit (the warp-level multi-split of Ashkiani et al.), a
// fixed cost; otherwise one __match_any_sync.
template <int RB, bool BALLOT>
__device__ __forceinline__ uint32_t same_digit_lanes(uint32_t d, bool valid) {
  if constexpr (BALLOT) {
    uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const bool bit = (d >> b) & 1u;
      const uint32_t bb = __ballot_sync(0xffffffffu, bit);
      peers &= bit ? bb : ~bb;
    }
    return peers;
  } else {
    return __match_any_sync(0xffffffffu, valid ? d : (1u << RB));
  }
}

// In view-major mode (view_shift > 0) a key is (view << view_shift) | local
// tile and the range goes to the view's global tile tile_offset + local.
__device__ __forceinline__ uint32_t range_slot(uint32_t key, uint32_t n_tiles,
                                               const gsx_batch_view *views, int32_t n_views,
                                               int view_shift) {
  if (!view_shift) return key < n_tiles ? key : 0xffffffffu;
  const uint32_t v = key >> view_shift, t = key & ((1u << view_shift) - 1u);
  if (v >= (uint32_t)n_views) return 0xffffffffu;
  const gsx_batch_view &vw = views[v];
  if ((int64_t)t >= (int64_t)vw.n_tiles_w * vw.n_tiles_h) return 0xffffffffu;
  return (uint32_t)(vw.tile_offset + t);
}

// Tile ranges written by the last tile pass (start == nullptr in every other
// pass): a pass's output is sorted, so each tile's keys are contiguous, and a
// key whose neighbour in its chunk's digit run holds another tile starts (or
// ends) its tile there, while a key at either end of a run may continue the
// tile of the neighbouring chunk: those positions go through atomicMin /
// atomicMax on start (all ones, the largest unsigned, until set) and end (-1).
struct RangeOut {
  int32_t *start, *end;
  const gsx_batch_view *views;
  int32_t n_views, view_shift;
  uint32_t n_tiles;
};

// Histogram of `passes` RB-bit digits (starting at bit 0) of n keys.
template <int RB>
__global__ void __launch_bounds__(kThreads)
    histogram_kernel(const uint32_t *__restrict__ keys, uint32_t n_max,
                     const uint32_t *__restrict__ n_dev, int passes,
                     uint32_t *__restrict__ hist) {
  constexpr uint32_t RADIX = 1u << RB, MASK = RADIX - 1u;
  __shared__ uint32_t sh[4 * 256];  // passes * RADIX <= 1024
  pdl_wait();
  pdl_trigger();
  const uint32_t n = n_dev ? min(*n_dev, n_max) : n_max;
  for (int i = threadIdx.x; i < 4 * 256; i += kThreads) sh[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const uint32_t k = keys[i];
    for (int p = 0; p < passes; ++p) atomicAdd(&sh[p * RADIX + ((k >> (RB * p)) & MASK)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * (int)RADIX; i += kThreads)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// One stable LSD pass on the RB-bit digit at `shift` (RB = 8 or 9), chunks
// of kThreads * ITEMS keys; thread t owns digits t*DPT .. t*DPT + DPT - 1.
// vals_in == nullptr means value = input position.  The item count is n_max,
// or *n_dev when given (a count produced on the device); chunks past it exit
// at once, and no chunk ever waits on a later one.  `status` holds RADIX
// look-back words per chunk.
template <int RB, int ITEMS, bool RANGES = false, bool BALLOT = false>
__global__ void __launch_bounds__(kThreads, 3)  // three CTAs per SM (shared memory allows three)
    onesweep_kernel(const uint32_t *__restrict__ keys_in,
                    const uint32_t *__restrict__ vals_in, uint32_t *__restrict__ keys_out,
                    uint32_t *__restrict__ vals_out, uint32_t n_max,
                    const uint32_t *__restrict__ n_dev, int shift,
                    const uint32_t *__restrict__ pass_hist, uint32_t *status,
                    uint32_t *chunk_counter, uint32_t *error, const RangeOut ro) {
  constexpr uint32_t RADIX = 1u << RB, MASK = RADIX - 1u;
  constexpr int DPT = (int)RADIX / kThreads;  // digits per thread
  constexpr int TILE = kThreads * ITEMS;
  static_assert(DPT >= 1 && DPT * kThreads == (int)RADIX, "RADIX must be a multiple of kThreads");
  pdl_wait();
  pdl_trigger();
  const uint32_t n = n_dev ? min(*n_dev, n_max) : n_max;
  __shared__ uint32_t s_warp[kWarps][RADIX];
  __shared__ uint32_t s_cta_excl[RADIX];
  __shared__ uint32_t s_glob[RADIX];
  __shared__ uint32_t s_tmp[kWarps];
  __shared__ uint32_t s_keys[TILE];
  __shared__ uint32_t s_vals[TILE];
  __shared__ uint32_t s_chunk;

  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  if (t == 0) s_chunk = atomicAdd(chunk_counter, 1u);
  for (int i = t; i < kWarps * (int)RADIX; i += kThreads) (&s_warp[0][0])[i] = 0;
  __syncthreads();
  const uint32_t chunk = s_chunk;
  const uint32_t base = chunk * (uint32_t)TILE;
  if (base >= n) return;  // block-uniform
  const uint32_t lt = lanemask_lt();

  uint32_t keys[ITEMS], vals[ITEMS], rank[ITEMS];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t idx = base + w * (32 * ITEMS) + j * 32 + lane;
    const bool valid = idx < n;
    const uint32_t k = valid ? keys_in[idx] : 0u;
    keys[j] = k;
    vals[j] = valid ? (vals_in ? vals_in[idx] : idx) : 0u;
    const uint32_t d = (k >> shift) & MASK;
    const uint32_t peers = same_digit_lanes<RB, BALLOT>(d, valid);
    uint32_t cnt = 0;
    if (valid) cnt = s_warp[w][d];
    __syncwarp();
    const uint32_t r = __popc(peers & lt);
    if (valid && r == 0) s_warp[w][d] = cnt + __popc(peers);
    rank[j] = cnt + r;
    __syncwarp();
  }
  __syncthreads();

  // per digit: exclusive prefix over warps, CTA total
  uint32_t total[DPT], hsum[DPT];
  uint32_t tsum = 0, hs = 0;
#pragma unroll
  for (int q = 0; q < DPT; ++q) {
    const int d = t * DPT + q;
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < kWarps; ++ww) {
      const uint32_t c = s_warp[ww][d];
      s_warp[ww][d] = run;
      run += c;
    }
    total[q] = run;
    tsum += run;
    hsum[q] = pass_hist[d];
    hs += hsum[q];
  }
  uint32_t cta_excl = block_exclusive_scan<uint32_t>(tsum, s_tmp, nullptr);
  uint32_t gbase = block_exclusive_scan<uint32_t>(hs, s_tmp, nullptr);

  // decoupled look-back for this thread's digits: publish every aggregate
  // first, then walk back
  uint32_t prev[DPT];
#pragma unroll
  for (int q = 0; q < DPT; ++q) {
    prev[q] = 0;
    uint32_t *mine = status + (size_t)chunk * RADIX + t * DPT + q;
    st_volatile(mine, (chunk == 0 ? kFlagPrefix : kFlagAgg) | total[q]);
  }
  if (chunk > 0) {
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
      const int d = t * DPT + q;
      int64_t c = (int64_t)chunk - 1;
      uint32_t spins = 0;
      while (c >= 0) {
        const uint32_t sv = ld_volatile(status + (size_t)c * RADIX + d);
        const uint32_t flag = sv & ~kCountMask;
        if (flag == 0u) {
          if (++spins > kSpinLimit) {
            atomicOr(error, kErrTimeout);
            break;
          }
          __nanosleep(32);
          continue;
        }
        prev[q] += sv & kCountMask;
        if (flag == kFlagPrefix) break;
        --c;
      }
      st_volatile(status + (size_t)chunk * RADIX + d, kFlagPrefix | (prev[q] + total[q]));
    }
  }
#pragma unroll
  for (int q = 0; q < DPT; ++q) {
    const int d = t * DPT + q;
    s_cta_excl[d] = cta_excl;
    s_glob[d] = gbase + prev[q];
    cta_excl += total[q];
    gbase += hsum[q];
  }
  __syncthreads();

#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t idx = base + w * (32 * ITEMS) + j * 32 + lane;
    if (idx < n) {
      const uint32_t d = (keys[j] >> shift) & MASK;
      const uint32_t pos = s_cta_excl[d] + s_warp[w][d] + rank[j];
      s_keys[pos] = keys[j];
      s_vals[pos] = vals[j];
    }
  }
  __syncthreads();
  const uint32_t cnt = min((uint32_t)TILE, n - base);
  for (uint32_t i = t; i < cnt; i += kThreads) {
    const uint32_t k = s_keys[i];
    const uint32_t d = (k >> shift) & MASK;
    const uint32_t g0 = s_cta_excl[d];
    const uint32_t gpos = s_glob[d] + (i - g0);
    if (gpos < n) {  // always true unless a look-back wait expired
      keys_out[gpos] = k;
      vals_out[gpos] = s_vals[i];
      if (RANGES) {
        const uint32_t g1 = d + 1 < RADIX ? s_cta_excl[d + 1] : cnt;  // end of the digit's run
        const bool head = i == g0, tail = i + 1 == g1;
        const bool first = head || s_keys[i - 1] != k;
        const bool last = tail || s_keys[i + 1] != k;
        if (first || last) {
          const uint32_t slot = range_slot(k, ro.n_tiles, ro.views, ro.n_views, ro.view_shift);
          if (slot != 0xffffffffu) {
            if (first) {
              if (head) atomicMin(reinterpret_cast<unsigned int *>(ro.start + slot), gpos);
              else ro.start[slot] = (int32_t)gpos;
            }
            if (last) {
              if (tail) atomicMax(ro.end + slot, (int32_t)(gpos + 1));
              else ro.end[slot] = (int32_t)(gpos + 1);
            }
          }
        }
      }
    }
  }
}

// Keys of one rectangle, capped at 2^31 (far above any key capacity) so the
// 62-bit scan cannot overflow for up to 2^30 Gaussians.
__device__ __forceinline__ long long rect_count(const int32_t *tl, const int32_t *br) {
  const long long w = (long long)br[0] - tl[0] + 1, h = (long long)br[1] - tl[1] + 1;
  if (w <= 0 || h <= 0) return 0;
  if (w >= (1ll << 31) || h >= (1ll << 31)) return 1ll << 31;
  const long long c = w * h;
  return c < (1ll << 31) ? c : (1ll << 31);
}

// Makes the depth order of a batch view-major: writes the view of every item
// in depth order as the key of one more stable pass, and clears the state
// that pass reuses from the first depth pass (its histogram row, chunk ticket
// and look-back rows), which the depth sort no longer needs.
__global__ void __launch_bounds__(kThreads)
    view_keys_kernel(const uint32_t *__restrict__ order, uint32_t n,
                     const gsx_batch_view *__restrict__ views, int32_t n_views,
                     uint32_t *__restrict__ vkeys, uint32_t *__restrict__ hist_row,
                     uint32_t *__restrict__ rows, uint32_t row_words, uint32_t *__restrict__ ticket) {
  __shared__ long long s_off[256];  // item offsets of the views (n_views <= 256)
  pdl_wait();
  pdl_trigger();
  for (int v = threadIdx.x; v < n_views; v += blockDim.x) s_off[v] = views[v].item_offset;
  __syncthreads();
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t i = first; i < n; i += stride) {
    const long long g = order[i];
    int lo = 0, hi = n_views - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_off[mid] <= g) lo = mid;
      else hi = mid - 1;
    }
    vkeys[i] = (uint32_t)lo;
  }
  for (uint32_t i = first; i < row_words; i += stride) rows[i] = 0u;
  if (first < 256) hist_row[first] = 0u;
  if (first == 0) *ticket = 0u;
}

// Exclusive scan of key counts in depth order (decoupled look-back over
// chunks of kEmitTile = 512 Gaussians) fused with the emission of (tile,
// Gaussian) pairs.  Warp w of a chunk owns its items w*64 + j*32 + lane
// (j = 0, 1), so item loads are coalesced; per group j the warp scans the 32
// counts and then writes the group's keys cooperatively, lane l taking keys
// l, l+32, ... of the group (the owner item found by a 5-step search), so key
// writes are coalesced too.  Chunks are small because the key count per
// Gaussian falls steeply with depth: the nearest chunks carry most keys, and
// smaller chunks spread them over more CTAs.  The last chunk writes the key
// total.
__global__ void __launch_bounds__(kThreads)
    emit_kernel(const uint32_t *__restrict__ order, uint32_t n,
                const int32_t *__restrict__ rect_tl, const int32_t *__restrict__ rect_br,
                int rect_stride, const int32_t *__restrict__ counts, int32_t n_tiles_w,
                int32_t n_tiles_h, const gsx_batch_view *__restrict__ views, int32_t n_views,
                uint32_t *__restrict__ tile_out, uint32_t *__restrict__ id_out,
                unsigned long long capacity, unsigned long long *status,
                uint32_t *chunk_counter, unsigned long long *total_out, uint32_t *k_eff,
                uint32_t *error, int view_shift) {
  __shared__ unsigned long long s_tmp[kWarps];
  __shared__ unsigned long long s_prefix;
  __shared__ uint32_t s_chunk;
  // staging of one 32-item group per warp
  __shared__ unsigned long long s_excl[kWarps][32];
  __shared__ uint32_t s_g[kWarps][32], s_tb[kWarps][32];
  __shared__ int32_t s_x0[kWarps][32], s_y0[kWarps][32], s_w[kWarps][32], s_ntw[kWarps][32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  pdl_wait();
  pdl_trigger();
  if (t == 0) s_chunk = atomicAdd(chunk_counter, 1u);
  __syncthreads();
  const uint32_t chunk = s_chunk;
  const uint32_t first = chunk * (uint32_t)kEmitTile + (uint32_t)w * (32 * kEmitItems) + lane;
  uint32_t gid[kEmitItems];
  long long cnt[kEmitItems];
  unsigned long long mysum = 0;
#pragma unroll
  for (int j = 0; j < kEmitItems; ++j) {
    const uint32_t idx = first + 32u * j;
    gid[j] = 0;
    cnt[j] = 0;
    if (idx < n) {
      const uint32_t g = order[idx];
      if (g >= n) {
        atomicOr(error, kErrIndex);
        continue;
      }
      gid[j] = g;
      const int32_t *tl = rect_tl + (size_t)g * rect_stride;
      const int32_t *br = rect_br + (size_t)g * rect_stride;
      const long long c = counts ? (long long)max(counts[g], 0) : rect_count(tl, br);
      cnt[j] = c;
      mysum += (unsigned long long)c;
    }
  }
  // warp totals -> offsets of the warps within the chunk, chunk total
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mysum += __shfl_xor_sync(0xffffffffu, mysum, o);
  if (lane == 0) s_tmp[w] = mysum;
  __syncthreads();
  unsigned long long warp_off = 0, block_total = 0;
#pragma unroll
  for (int k = 0; k < kWarps; ++k) {
    const unsigned long long c = s_tmp[k];
    if (k < w) warp_off += c;
    block_total += c;
  }
  if (w == 0) {
    // decoupled look-back, 32 predecessors per poll: lane l reads chunk
    // c - l; the nearest inclusive prefix ends the walk, the aggregates of
    // the chunks before it are summed with the prefix.
    unsigned long long prev = 0;
    unsigned long long *mine = status + chunk;
    if (chunk == 0) {
      if (lane == 0) st_volatile64(mine, kFlag64Prefix | block_total);
    } else {
      if (lane == 0) st_volatile64(mine, kFlag64Agg | block_total);
      int64_t c = (int64_t)chunk - 1;
      uint32_t spins = 0;
      while (true) {
        const int64_t idx = c - lane;
        const unsigned long long sv = idx >= 0 ? ld_volatile64(status + idx) : kFlag64Prefix;
        const unsigned long long flag = sv & ~kCount64Mask;
        const uint32_t pmask = __ballot_sync(0xffffffffu, flag == kFlag64Prefix);
        const uint32_t zmask = __ballot_sync(0xffffffffu, flag == 0ull);
        const int first = pmask ? __ffs(pmask) - 1 : 31;  // last lane the walk needs
        const uint32_t need = first == 31 ? 0xffffffffu : ((2u << first) - 1u);
        if (zmask & need) {  // a needed predecessor has not published yet
          if (++spins > kSpinLimit) {
            if (lane == 0) atomicOr(error, kErrTimeout);
            break;
          }
          __nanosleep(32);
          continue;
        }
        unsigned long long v = lane <= first ? (sv & kCount64Mask) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        prev += v;
        if (pmask) break;
        c -= 32;
      }
      if (lane == 0) st_volatile64(mine, kFlag64Prefix | (prev + block_total));
    }
    if (lane == 0) {
      s_prefix = prev;
      if ((unsigned long long)(chunk + 1) * kEmitTile >= n) {
        const unsigned long long total = prev + block_total;
        *total_out = total;
        *k_eff = (uint32_t)(total < capacity ? total : capacity);
      }
    }
  }
  __syncthreads();
  unsigned long long gbase = s_prefix + warp_off;  // first key of the current group
#pragma unroll
  for (int j = 0; j < kEmitItems; ++j) {
    // group scan: exclusive offsets of the 32 items, group total
    unsigned long long x = (unsigned long long)cnt[j];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const unsigned long long gtotal = __shfl_sync(0xffffffffu, x, 31);
    const unsigned long long excl = x - (unsigned long long)cnt[j];
    int32_t x0 = 0, y0 = 0, wd = 1, ntw = n_tiles_w;
    uint32_t tile_base = 0xffffffffu;  // all ones: the item lies outside its tile grid
    if (cnt[j] > 0) {
      const uint32_t g = gid[j];
      const int32_t *tl = rect_tl + (size_t)g * rect_stride;
      const int32_t *br = rect_br + (size_t)g * rect_stride;
      if (rect_count(tl, br) != cnt[j]) atomicOr(error, kErrCount);
      // tiles of this item's image: one image, or the item's view in a batch
      int32_t nth = n_tiles_h;
      uint32_t tb = 0;
      if (views) {
        int lo = 0, hi = n_views - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (views[mid].item_offset <= (int64_t)g) lo = mid;
          else hi = mid - 1;
        }
        ntw = views[lo].n_tiles_w;
        nth = views[lo].n_tiles_h;
        // global tile ids, or (view << view_shift) | local tile in view-major mode
        tb = view_shift ? (uint32_t)lo << view_shift : (uint32_t)views[lo].tile_offset;
      }
      const bool in_grid = tl[0] >= 0 && tl[1] >= 0 && br[0] < ntw && br[1] < nth;
      if (!in_grid) atomicOr(error, kErrRange);
      else tile_base = tb;
      x0 = tl[0];
      y0 = tl[1];
      wd = max(br[0] - tl[0] + 1, 1);
    }
    s_excl[w][lane] = excl;
    s_g[w][lane] = gid[j];
    s_tb[w][lane] = tile_base;
    s_x0[w][lane] = x0;
    s_y0[w][lane] = y0;
    s_w[w][lane] = wd;
    s_ntw[w][lane] = ntw;
    __syncwarp();
    // keys [gbase, gbase + gtotal) of which those below the capacity are written
    const unsigned long long lim =
        gbase >= capacity ? 0ull : (gtotal < capacity - gbase ? gtotal : capacity - gbase);
    for (unsigned long long q = lane; q < lim; q += 32) {
      int lo = 0, hi = 31;
#pragma unroll
      for (int step = 0; step < 5; ++step) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_excl[w][mid] <= q) lo = mid;
        else hi = mid - 1;
      }
      const uint32_t local = (uint32_t)(q - s_excl[w][lo]);
      const uint32_t wdt = (uint32_t)s_w[w][lo];
      const uint32_t ry = local / wdt, rx = local - ry * wdt;
      const uint32_t tb = s_tb[w][lo];
      const unsigned long long pos = gbase + q;
      tile_out[pos] = tb == 0xffffffffu
                          ? 0xffffffffu
                          : tb + (uint32_t)(((int32_t)ry + s_y0[w][lo]) * s_ntw[w][lo] +
                                            ((int32_t)rx + s_x0[w][lo]));
      id_out[pos] = s_g[w][lo];
    }
    __syncwarp();
    gbase += gtotal;
  }
}

// start/end of every tile from the sorted tile ids: 4 consecutive keys per
// thread (one 16-byte load; `tiles` is 16-byte aligned), their neighbours
// from the adjacent threads' loads or, at warp edges, from memory.
__global__ void ranges_kernel(const uint32_t *__restrict__ tiles, const uint32_t *__restrict__ K_dev,
                              uint32_t n_tiles, int32_t *__restrict__ start,
                              int32_t *__restrict__ end, const gsx_batch_view *__restrict__ views,
                              int32_t n_views, int view_shift) {
  pdl_wait();
  pdl_trigger();
  const uint32_t K = *K_dev;
  const uint32_t base = 4u * (blockIdx.x * blockDim.x + threadIdx.x);
  if (base >= K) return;
  uint32_t v[4];
  if (base + 4 <= K) {
    const uint4 q = *reinterpret_cast<const uint4 *>(tiles + base);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = base + j < K ? tiles[base + j] : 0xffffffffu;
  }
  const uint32_t prev = base > 0 ? tiles[base - 1] : 0xffffffffu;
  const uint32_t next = base + 4 < K ? tiles[base + 4] : 0xffffffffu;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint32_t i = base + j;
    if (i >= K) break;
    const uint32_t t = v[j];
    const uint32_t before = j == 0 ? prev : v[j - 1];
    const uint32_t after = j == 3 ? next : v[j + 1];
    const bool first_key = i == 0 || before != t, last_key = i == K - 1 || after != t;
    if (!first_key && !last_key) continue;
    const uint32_t slot = range_slot(t, n_tiles, views, n_views, view_shift);
    if (slot == 0xffffffffu) continue;
    if (first_key) start[slot] = (int32_t)i;
    if (last_key) end[slot] = (int32_t)(i + 1);
  }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Binning workspace.  Everything that must start at zero -- the chunk
// tickets, the status block, the digit histograms and every pass's look-back
// flags -- sits in one contiguous region (`zero_begin`, cleared by a single
// memset per call up to the last pass in use); each pass owns its own
// look-back flags and ticket, so nothing is cleared between passes.
constexpr int kMaxPasses = 4;  // 8-bit digits of a 32-bit key
struct Workspace {
  uint32_t *dkeys[2], *dvals[2];
  uint32_t *tkeys[2], *tvals[2];
  char *zero_begin;
  uint32_t *counters;  // [16]: depth passes 0-3, tile passes 4-7, emission 8
  uint32_t *error;
  unsigned long long *total;
  uint32_t *k_eff;  // min(total, capacity), the key count the tile sort uses
  uint32_t *hist;   // [8][256]: depth digits 0-3, tile digits 4-7
  unsigned long long *emit_status;
  uint32_t *status_depth;  // [kMaxPasses][depth_chunks][256]
  uint32_t *status_tile;   // [kMaxPasses][tile_chunks][256]
  size_t depth_chunks, tile_chunks, emit_words;
  size_t bytes;
};

Workspace carve_ws(void *base, int64_t n, int64_t cap) {
  Workspace w;
  char *p = static_cast<char *>(base);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *r = p ? p + off : nullptr;
    off += align256(bytes);
    return r;
  };
  const size_t nn = (size_t)(n > 0 ? n : 1), cc = (size_t)(cap > 0 ? cap : 1);
  for (int i = 0; i < 2; ++i) w.dkeys[i] = reinterpret_cast<uint32_t *>(take(4 * nn));
  for (int i = 0; i < 2; ++i) w.dvals[i] = reinterpret_cast<uint32_t *>(take(4 * nn));
  for (int i = 0; i < 2; ++i) w.tkeys[i] = reinterpret_cast<uint32_t *>(take(4 * cc));
  for (int i = 0; i < 2; ++i) w.tvals[i] = reinterpret_cast<uint32_t *>(take(4 * cc));
  // zero-initialised region, in the order the passes use it
  w.zero_begin = take(0);
  w.counters = reinterpret_cast<uint32_t *>(take(16 * 4));
  // the status block: key total (u64), error bits (u32), key count used (u32),
  // 16 contiguous bytes that one copy brings back
  char *status_block = take(kStatusBlockBytes);
  w.total = reinterpret_cast<unsigned long long *>(status_block);
  w.error = reinterpret_cast<uint32_t *>(status_block ? status_block + 8 : nullptr);
  w.k_eff = reinterpret_cast<uint32_t *>(status_block ? status_block + 12 : nullptr);
  w.hist = reinterpret_cast<uint32_t *>(take(8 * 256 * 4));
  w.emit_words = (nn + kEmitTile - 1) / kEmitTile;
  w.emit_status = reinterpret_cast<unsigned long long *>(take(8 * w.emit_words));
  w.depth_chunks = (nn + kTile - 1) / kTile;
  w.status_depth = reinterpret_cast<uint32_t *>(take(4 * 256 * kMaxPasses * w.depth_chunks));
  w.tile_chunks = (cc + kTileMin - 1) / kTileMin;
  w.status_tile = reinterpret_cast<uint32_t *>(take(4 * 256 * kMaxPasses * w.tile_chunks));
  w.bytes = off;
  return w;
}

// Digit width and pass count of an LSD sort over `bits` key bits: 8-bit
// digits, except that 17-18 bits take two 9-bit passes instead of three.
inline int digit_bits(int bits) { return (bits == 17 || bits == 18) ? 9 : 8; }
inline int sort_passes(int bits) { return (bits + digit_bits(bits) - 1) / digit_bits(bits); }

// Stable LSD sort of n (key, value) pairs over `bits` low key bits; the count
// is n_max, or *n_dev (at most n_max) when n_dev is given.  The final pass
// writes into (final_keys, final_vals); intermediate passes use the two
// scratch buffers.  keys_in/vals_in are never written.  `hist` (up to 1024
// digit counts), `tickets` (one chunk counter per pass) and `status` (per
// pass, `chunks_cap` rows of 2^digit_bits look-back words) must be zero on
// entry.
int radix_sort(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t n_max,
               const uint32_t *n_dev, int bits, uint32_t *scratch_k[2], uint32_t *scratch_v[2],
               uint32_t *final_keys, uint32_t *final_vals, uint32_t *hist, uint32_t *tickets,
               uint32_t *status, size_t chunks_cap, uint32_t *error, cudaStream_t s,
               const RangeOut ranges = RangeOut{}) {
  const int rb = digit_bits(bits), passes = sort_passes(bits);
  // digit matching by ballots for lists up to 32 Mi keys, by __match_any_sync
  // above: measured, the 1M-key depth passes and 4M-key tile passes of one
  // 1080p view ran faster with ballots (binning 0.276 -> 0.265 ms), the
  // 181M-key tile passes of a 32-view batch slower (5.25 -> 5.72 ms)
  const bool ballot = n_max <= (32u << 20);
  if (n_max == 0 || bits == 0) return GSX_OK;
  const uint32_t radix = 1u << rb;
  uint32_t hist_grid = (n_max + kThreads * 16 - 1) / (kThreads * 16);
  if (hist_grid > 1024u) hist_grid = 1024u;
  count_launches(1);
  cudaError_t e =
      rb == 9 ? launch_pdl(histogram_kernel<9>, hist_grid, kThreads, 0, s, keys_in, n_max, n_dev, passes, hist)
              : launch_pdl(histogram_kernel<8>, hist_grid, kThreads, 0, s, keys_in, n_max, n_dev, passes, hist);
  if (e != cudaSuccess) return cuda_status(e, "histogram_kernel launch");
  const uint32_t tile = kThreads * (rb == 9 ? kItems9 : kItems);
  const uint32_t chunks = (n_max + tile - 1) / tile;
  // rows are laid out for 256-word digits: a 512-word pass takes two rows' room
  if ((size_t)chunks * radix * passes > chunks_cap * 256 * 4) {
    set_error("radix sort of %u keys needs %u chunks, the workspace holds %zu", n_max, chunks,
              chunks_cap);
    return GSX_ERR_CAPACITY;
  }
  const uint32_t *ki = keys_in, *vi = vals_in;
  for (int p = 0; p < passes; ++p) {
    const bool last = p == passes - 1;
    uint32_t *ko = last ? final_keys : scratch_k[p & 1];
    uint32_t *vo = last ? final_vals : scratch_v[p & 1];
    uint32_t *st = status + (size_t)chunks * radix * p;
    count_launches(1);
    const bool rng = last && ranges.start;
    const RangeOut ro = rng ? ranges : RangeOut{};
    auto k9 = rng ? onesweep_kernel<9, kItems9, true> : onesweep_kernel<9, kItems9, false>;
    auto k8 = rng ? (ballot ? onesweep_kernel<8, kItems, true, true> : onesweep_kernel<8, kItems, true>)
                  : (ballot ? onesweep_kernel<8, kItems, false, true> : onesweep_kernel<8, kItems, false>);
    e = rb == 9 ? launch_pdl(k9, chunks, kThreads, 0, s, ki, vi, ko, vo, n_max, n_dev, rb * p, hist + radix * p, st,
                             tickets + p, error, ro)
                : launch_pdl(k8, chunks, kThreads, 0, s, ki, vi, ko, vo, n_max, n_dev, rb * p, hist + radix * p, st,
                             tickets + p, error, ro);
    if (e != cudaSuccess) return cuda_status(e, "onesweep_kernel launch");
    ki = ko;
    vi = vo;
  }
  return GSX_OK;
}

int bits_for(uint64_t max_value) {
  int b = 0;
  while (b < 32 && (max_value >> b) != 0) ++b;
  return b;
}

}  // namespace

size_t binning_workspace_bytes(int64_t n, int64_t cap, int64_t n_tiles) {
  (void)n_tiles;
  return carve_ws(nullptr, n, cap).bytes;
}

// Diagnostic of the look-back's bounded wait: one onesweep pass of 2 chunks
// launched as a single CTA whose ticket is preset to 1, so it claims chunk 1
// and waits for chunk 0, which no CTA ever publishes.  The wait gives up after
// its poll limit, sets the timeout bit and the CTA finishes its pass.
// `scratch` (>= look_back_selftest_bytes()) is caller device memory; returns
// the binning status the timeout maps to (GSX_ERR_TIMEOUT when it works).
size_t look_back_selftest_bytes() { return align256(4 * (size_t)kTile * 2 * 4) + 4 * 256 * 2 * 2 + 64; }

int look_back_selftest(void *scratch, size_t bytes, uint32_t *error_host, cudaStream_t s) {
  if (bytes < look_back_selftest_bytes()) {
    set_error("self-test scratch too small: %zu < %zu bytes", bytes, look_back_selftest_bytes());
    return GSX_ERR_CAPACITY;
  }
  if ((reinterpret_cast<uintptr_t>(scratch) & 255) != 0) {
    set_error("self-test scratch must be 256-byte aligned");
    return GSX_ERR_INVALID_ARG;
  }
  const uint32_t n = 2 * kTile;
  char *p = static_cast<char *>(scratch);
  uint32_t *keys_in = reinterpret_cast<uint32_t *>(p);
  uint32_t *keys_out = keys_in + n, *vals_in = keys_in + 2 * n, *vals_out = keys_in + 3 * n;
  char *state = p + align256(4 * (size_t)n * 4);
  uint32_t *hist = reinterpret_cast<uint32_t *>(state);          // [256]
  uint32_t *status = hist + 256;                                 // [2 chunks][256]
  uint32_t *ticket = status + 2 * 256, *error = ticket + 1;
  cudaError_t e = cudaMemsetAsync(p, 0, look_back_selftest_bytes(), s);
  const uint32_t one = 1;
  // the histogram of 2*kTile zero keys: all in digit 0
  const uint32_t h0 = n;
  if (e == cudaSuccess) e = cudaMemcpyAsync(ticket, &one, 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hist, &h0, 4, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "look-back self-test set-up");
  count_launches(1);
  onesweep_kernel<8, kItems><<<1, kThreads, 0, s>>>(keys_in, vals_in, keys_out, vals_out, n, nullptr, 0, hist,
                                                     status, ticket, error, RangeOut{});
  e = cudaGetLastError();
  uint32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, error, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "look-back self-test");
  if (error_host) *error_host = err;
  return decode_binning_status(0, err, 0, 1, 1);
}

// Enqueue the whole binning on `s` without synchronising.  Keys beyond
// `capacity` are not written; the key total and the error bits stay in the
// workspace for binning_status.
int run_binning_async(int64_t n, const int32_t *rect_tl, const int32_t *rect_br,
                      int32_t rect_stride, const int32_t *counts, const float *depth,
                      int32_t n_tiles_w, int32_t n_tiles_h, int64_t capacity, int32_t *ids,
                      int32_t *start, int32_t *end, void *ws, size_t ws_bytes, cudaStream_t s,
                      const gsx_batch_view *views, int32_t n_views, int64_t total_tiles,
                      int64_t max_view_tiles) {
  const int64_t n_tiles = views ? total_tiles : (int64_t)n_tiles_w * n_tiles_h;
  Workspace w = carve_ws(ws, n, capacity);
  if (ws_bytes < w.bytes) {
    set_error("binning workspace too small: %zu < %zu bytes", ws_bytes, w.bytes);
    return GSX_ERR_CAPACITY;
  }
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0) {  // the kernels use 16-byte vector loads
    set_error("binning workspace must be 256-byte aligned");
    return GSX_ERR_INVALID_ARG;
  }
  // View-major batches (up to 256 views): one more stable pass orders the
  // depth-sorted items by view, the emitted keys are (view << view_shift) |
  // local tile, and the tile sort needs only the local bits (two 8-bit passes
  // for 1080p views at 16x16 instead of two 9-bit passes over the global ids):
  // a stable sort of view-major keys on their low bits keeps each (view, tile)
  // list contiguous and in depth order.
  int view_shift = 0;
  if (views && n_views <= 256 && max_view_tiles > 0) {
    const int lb = std::max(1, bits_for((uint64_t)(max_view_tiles - 1)));
    if (lb + bits_for((uint64_t)(n_views - 1)) <= 31) view_shift = lb;
  }
  const int tile_bits = view_shift ? view_shift : bits_for((uint64_t)(n_tiles > 0 ? n_tiles - 1 : 0));
  const int tile_passes = tile_bits == 0 ? 0 : sort_passes(tile_bits);
  // one clear of the zero-initialised state, through the last tile pass in
  // use (a pass's rows are packed: chunks x 2^digit_bits words)
  const uint32_t tile_chunk_keys = kThreads * (digit_bits(tile_bits) == 9 ? kItems9 : kItems);
  const size_t tile_rows = ((size_t)(capacity > 0 ? capacity : 1) + tile_chunk_keys - 1) / tile_chunk_keys;
  const char *zero_end = reinterpret_cast<const char *>(w.status_tile) +
                         (size_t)4 * tile_rows * ((size_t)1 << digit_bits(tile_bits)) * tile_passes;
  cudaError_t e = cudaMemsetAsync(start, 0xff, sizeof(int32_t) * (size_t)n_tiles, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(end, 0xff, sizeof(int32_t) * (size_t)n_tiles, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.zero_begin, 0, (size_t)(zero_end - w.zero_begin), s);
  if (e != cudaSuccess) return cuda_status(e, "memset binning state");
  if (n == 0) return GSX_OK;
  const uint32_t nn = (uint32_t)n;
  // 1. Gaussians sorted by depth bits (values = Gaussian index)
  uint32_t *sk[2] = {w.dkeys[0], w.dkeys[1]}, *sv[2] = {w.dvals[0], w.dvals[1]};
  int st = radix_sort(reinterpret_cast<const uint32_t *>(depth), nullptr, nn, nullptr, 32, sk, sv,
                      w.dkeys[1], w.dvals[1], w.hist, w.counters, w.status_depth, w.depth_chunks,
                      w.error, s);
  if (st != GSX_OK) return st;
  const uint32_t *order = w.dvals[1];
  if (view_shift && n_views > 1) {
    // 1b. stable pass on the view of each item: (view, depth) order.  The
    // depth sort's first-pass state (histogram row, ticket, look-back rows)
    // is cleared by view_keys_kernel and reused; keys in dkeys[0], result in
    // dvals[0] (its keys in dkeys[1]).
    const uint32_t rows = (uint32_t)(((nn + kTile - 1) / kTile) * 256);
    const uint32_t grid = std::min<uint32_t>((nn + kThreads - 1) / kThreads, 4096u);
    count_launches(1);
    e = launch_pdl(view_keys_kernel, std::max(grid, 1u), kThreads, 0, s, (const uint32_t *)w.dvals[1], nn, views,
                   n_views, w.dkeys[0], w.hist, w.status_depth, rows, w.counters);
    if (e != cudaSuccess) return cuda_status(e, "view_keys_kernel launch");
    uint32_t *vk[2] = {w.dkeys[1], w.dkeys[1]}, *vv[2] = {w.dvals[0], w.dvals[0]};  // one pass: unused
    st = radix_sort(w.dkeys[0], w.dvals[1], nn, nullptr, bits_for((uint64_t)(n_views - 1)), vk, vv, w.dkeys[1],
                    w.dvals[0], w.hist, w.counters, w.status_depth, w.depth_chunks, w.error, s);
    if (st != GSX_OK) return st;
    order = w.dvals[0];
  }
  // 2. scan of counts + emission
  const uint32_t emit_chunks = (nn + kEmitTile - 1) / kEmitTile;
  count_launches(1);
  e = launch_pdl(emit_kernel, emit_chunks, kThreads, 0, s, order, nn, rect_tl, rect_br, rect_stride, counts,
                 n_tiles_w, n_tiles_h, views, n_views, w.tkeys[0], w.tvals[0], (unsigned long long)capacity,
                 w.emit_status, w.counters + 8, w.total, w.k_eff, w.error, view_shift);
  if (e != cudaSuccess) return cuda_status(e, "emit_kernel launch");
  if (capacity == 0) return GSX_OK;
  const uint32_t cap = (uint32_t)capacity;
  // 3. stable sort by tile id over the device-side key count.  Pass p writes
  // tkeys[1] for even p and tkeys[0] for odd p; the last pass writes the ids
  // into the caller's buffer and its keys into whichever tile buffer is not
  // its input.
  uint32_t *ids_u = reinterpret_cast<uint32_t *>(ids);
  uint32_t *final_keys = w.tkeys[0];
  if (tile_bits == 0) {
    e = cudaMemcpyAsync(ids_u, w.tvals[0], 4 * (size_t)cap, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_status(e, "copy ids");
  } else {
    const int passes = sort_passes(tile_bits);
    uint32_t *tk[2] = {w.tkeys[1], w.tkeys[0]}, *tv[2] = {w.tvals[1], w.tvals[0]};
    final_keys = (passes & 1) ? w.tkeys[1] : w.tkeys[0];
    // 4. start / end, written by the last pass
    const RangeOut ro{start, end, views, n_views, view_shift, (uint32_t)n_tiles};
    st = radix_sort(w.tkeys[0], w.tvals[0], cap, w.k_eff, tile_bits, tk, tv, final_keys, ids_u,
                    w.hist + 4 * 256, w.counters + 4, w.status_tile, w.tile_chunks, w.error, s, ro);
    return st;
  }
  // 4. start / end of a single tile
  count_launches(1);
  e = launch_pdl(ranges_kernel, (cap + 1023) / 1024, 256, 0, s, final_keys, w.k_eff, (uint32_t)n_tiles, start,
                 end, views, n_views, view_shift);
  if (e != cudaSuccess) return cuda_status(e, "ranges_kernel launch");
  return GSX_OK;
}

// Turn a copied status block (key total, error bits) into a status.
int decode_binning_status(unsigned long long total_h, uint32_t err_h, int64_t capacity,
                          int32_t n_tiles_w, int32_t n_tiles_h) {
  if (err_h & kErrTimeout) {
    set_error("binning: a look-back wait expired");
    return GSX_ERR_TIMEOUT;
  }
  if (err_h & kErrCount) {
    set_error("binning: key counts disagree with the rectangles");
    return GSX_ERR_MISMATCH;
  }
  if (err_h & kErrRange) {
    set_error("binning: a rectangle lies outside the %d x %d tile grid", n_tiles_w, n_tiles_h);
    return GSX_ERR_INVALID_ARG;
  }
  if (err_h & kErrIndex) {
    set_error("binning: corrupted depth order");
    return GSX_ERR_TIMEOUT;
  }
  if ((int64_t)total_h > capacity) {
    set_error("binning: %llu keys exceed the capacity of %lld", total_h, (long long)capacity);
    return GSX_ERR_CAPACITY;
  }
  return GSX_OK;
}

// Enqueue a copy of the status block left by run_binning_async into dst
// (16 bytes of pinned host or device memory); no synchronisation.
int copy_binning_status_async(const void *ws, int64_t n, int64_t capacity, void *dst,
                              cudaStream_t s) {
  Workspace w = carve_ws(const_cast<void *>(ws), n, capacity);
  cudaError_t e = cudaMemcpyAsync(dst, w.total, kStatusBlockBytes, cudaMemcpyDefault, s);
  return e == cudaSuccess ? GSX_OK : cuda_status(e, "copy binning status");
}

// Read the key total and error bits left by run_binning_async (synchronises
// `s`) and turn them into a status.
int binning_status(const void *ws, int64_t n, int64_t capacity, int32_t n_tiles_w,
                   int32_t n_tiles_h, int64_t *n_keys_host, uint32_t *flags_host,
                   cudaStream_t s) {
  Workspace w = carve_ws(const_cast<void *>(ws), n, capacity);
  uint64_t block[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(block, w.total, kStatusBlockBytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "read binning status");
  const unsigned long long total_h = block[0];
  const uint32_t err_h = (uint32_t)(block[1] & 0xffffffffu);
  if (n_keys_host) *n_keys_host = (int64_t)total_h;
  if (flags_host) *flags_host = err_h;
  return decode_binning_status(total_h, err_h, capacity, n_tiles_w, n_tiles_h);
}

int run_binning(int64_t n, const int32_t *rect_tl, const int32_t *rect_br,
                int32_t rect_stride, const int32_t *counts, const float *depth,
                int32_t n_tiles_w, int32_t n_tiles_h, int64_t capacity, int32_t *ids,
                int32_t *start, int32_t *end, int64_t *n_keys_host, void *ws,
                size_t ws_bytes, cudaStream_t s) {
  int st = run_binning_async(n, rect_tl, rect_br, rect_stride, counts, depth, n_tiles_w,
                             n_tiles_h, capacity, ids, start, end, ws, ws_bytes, s);
  if (st != GSX_OK) return st;
  return binning_status(ws, n, capacity, n_tiles_w, n_tiles_h, n_keys_host, nullptr, s);
}

}  // namespace gsx
