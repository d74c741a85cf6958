// Persistent work-stealing schedule of the mixed-precision multifit (the
// uneven ECAL 10x10 / HCAL 8x8 batches).
//
// The grid schedule (fit_mixed.cu) launches one thread per channel of the chunk
// for every condition set, so in a mixed batch the lanes of the other set idle
// through each launch; on this GPU an FP64 warp instruction costs its full pipe
// time whatever the number of active lanes, so the FP64 judge of a 60/40 batch
// runs at ~60 % lane efficiency. Here:
//
//   partition_kernel  one pass over ctype: per-set channel lists (warp-aggregated
//                     atomics, one per set present in a warp), out-of-range sets
//                     flagged BADINPUT (skipped for a batch without ctype, whose
//                     list is the identity);
//   search_persist    FP32 search over a set's list, L lanes per channel
//                     (32 / L channels per warp), each warp taking the next
//                     32 / L channels from an atomic counter when it is done;
//   screen_persist    (cold starts) FP32 double-float KKT screen over the list;
//   judge_persist     FP64 (or double-float) judge over the list, 32 channels
//                     per steal;
//   fix_persist       FP32 FNNLS step of the channels the screen or (warm
//                     starts) the judge queued for it;
//   judge_fixed_persist  (warm starts) the judge again on those;
//   repair_persist    FP64 repair over the judge's queue, 32 per steal.
//
// Grids are sized from the occupancy of each kernel (blocks per SM x SMs), so
// every launch is one wave of resident warps that drains its list. The
// per-channel arithmetic is the grid schedule's (mixed_device.cuh); for L > 1
// only the passive-set solves are split over the lanes of a channel (each lane
// takes the samples i = sub (mod L) and the partial sums meet in a butterfly),
// every other step runs redundantly and identically in the L lanes.
#include <mutex>

#include "mixed_device.cuh"

namespace mfgb {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// ws_sched words
constexpr int SCHED_COUNT = 0;   // [set] channels in the set's list
constexpr int SCHED_STEAL = 2;   // [set * 6 + kernel] work counters (search, second judge, fix, judge, repair,
                                 // screen)
constexpr int SCHED_QUEUE = 14;  // [set] channels queued for repair
constexpr int SCHED_FIXQ = 16;   // [set] channels queued by the screen or the judge for the fix

__global__ void partition_kernel(const MixedArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t base = int64_t(blockIdx.x) * blockDim.x; base < a.n; base += stride) {
    const int64_t ch = base + threadIdx.x;
    const bool in = ch < a.n;
    int t = -1;
    if (in) {
      t = a.ctype ? int(a.ctype[ch]) : 0;
      if (t >= a.n_ctypes) {
        if (a.status) a.status[ch] = CH_BADINPUT;
        a.chi2[ch] = 0.;
        t = -1;
      }
    }
    // lanes of one set append together: one atomic per set present in the warp
    const unsigned peers = __match_any_sync(kFull, t);
    if (t >= 0) {
      const int leader = __ffs(peers) - 1;
      unsigned pos = 0;
      if (lane == leader) pos = atomicAdd(a.ws_sched + SCHED_COUNT + t, unsigned(__popc(peers)));
      pos = __shfl_sync(peers, pos, leader);
      a.ws_list[int64_t(t) * MIXED_CHUNK + pos + __popc(peers & ((1u << lane) - 1u))] = int(ch);
    }
  }
}

// Passive-set solve of the cooperative search: lane `sub` of the channel's L
// lanes sums the samples i = sub + L q; the butterfly leaves the same sum in
// all L lanes (each level adds the same two values in either order).
template <int N, int K, int L>
__device__ __forceinline__ void solve32_coop(const DevMixed& T, unsigned m, const float* yo, int sub, unsigned gmask,
                                             float* s) {
  constexpr int Q = (N + L - 1) / L;
  const float* P = T.pinv32 + __ldg(T.offset + m);
  int r = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float acc = 0.f;
    if (m & (1u << k)) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int i = sub + L * q;
        if (i < N) acc = fmaf(__ldg(P + r * N + i), yo[q], acc);
      }
      ++r;
    }
#pragma unroll
    for (int off = L / 2; off >= 1; off /= 2) acc += __shfl_xor_sync(gmask, acc, off);
    s[k] = acc;
  }
}

// The FP32 search of channel ch by its L lanes (lane `sub` of the group).
// Same steps as search_body; the passive-set solves are split over the lanes.
template <int N, int K, int L, bool WARM>
__device__ __forceinline__ void search_body_coop(const MixedArgs& a, const DevMixed& T, int64_t ch, int sub,
                                                 unsigned gmask) {
  constexpr int Q = (N + L - 1) / L;
  const double* in = a.samples + ch * a.sample_stride;
  float sf[N], y32[N], ynorm2 = 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i) sf[i] = float(in[i]);
  {
    int w = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      float acc = 0.f;
#pragma unroll
      for (int j = 0; j <= i; ++j) acc = fmaf(T.W32[w + j], sf[j], acc);
      w += i + 1;
      y32[i] = acc;
      ynorm2 = fmaf(acc, acc, ynorm2);
    }
  }
  float yo[Q];  // this lane's samples i = sub + L q
#pragma unroll
  for (int q = 0; q < Q; ++q) yo[q] = 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (i % L == sub) yo[i / L] = y32[i];
  float c32[K];
  gram_rhs32<N, K>(T, y32, c32, nullptr);
  const float ynorm = sqrtf(ynorm2);
  const unsigned full = (1u << K) - 1u;
  unsigned m = 0;
  float x32[K];
#pragma unroll
  for (int k = 0; k < K; ++k) x32[k] = 0.f;
  int adds = 0, solves = 0;
  auto s32 = [&](unsigned mm, float* out) { solve32_coop<N, K, L>(T, mm, yo, sub, gmask, out); };
  if (WARM) {
    m = unsigned(a.warm_mask[ch]) & full;
    const float* wa = a.warm_amp + ch * a.warm_stride;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (m & (1u << k)) x32[k] = fmaxf(wa[k], 1e-30f);
    if (m) solves += inner_loop<K>(m, x32, s32);
  }
  const int iters = WARM ? kWarmSearchIters : a.max_iter32;
  for (int it = 0; it < iters; ++it) {
    float wmax = 0.f;
    int imax = -1;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (m & (1u << k)) continue;
      float acc = c32[k];
#pragma unroll
      for (int j = 0; j < K; ++j) acc = fmaf(-T.H32[k * KMAX + j], x32[j], acc);
      const float tol = a.tol32 * T.gnorm32[k] * ynorm;
      if (acc > tol && (imax < 0 || acc > wmax)) {
        wmax = acc;
        imax = k;
      }
    }
    if (imax < 0) break;
    m |= 1u << imax;
    ++adds;
    solves += inner_loop<K>(m, x32, s32);
  }
  if (sub == 0) {
    a.ws_mask[ch] = uint16_t(m);
    a.ws_count[ch] = uint16_t((adds < 255 ? adds : 255) | ((solves < 255 ? solves : 255) << 8));
    float* wx = a.ws_x + ch * K;
#pragma unroll
    for (int k = 0; k < K; ++k) wx[k] = x32[k];
  }
}

// A warp's next unit of work: `per` consecutive list entries from the counter.
__device__ __forceinline__ unsigned steal(unsigned* counter, unsigned per) {
  unsigned base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(counter, per);
  return __shfl_sync(kFull, base, 0);
}

template <int N, int K, int L, bool WARM>
__global__ void __launch_bounds__(512) search_persist(const MixedArgs a, int set) {
  constexpr unsigned G = 32 / L;  // channels per warp
  const DevMixed& T = a.tab[set];
  const unsigned total = a.list_identity ? unsigned(a.n) : a.ws_sched[SCHED_COUNT + set];
  const int* list = a.ws_list + int64_t(set) * MIXED_CHUNK;
  const int lane = threadIdx.x & 31, sub = lane % L;
  const unsigned gmask = L == 32 ? kFull : (((1u << L) - 1u) << (lane - sub));
  for (;;) {
    const unsigned base = steal(a.ws_sched + SCHED_STEAL + set * 6 + 0, G);
    if (base >= total) break;
    const unsigned i = base + unsigned(lane / L);
    if (i < total) {
      const int64_t ch = a.list_identity ? int64_t(i) : int64_t(list[i]);
      if constexpr (L == 1) search_body<N, K, WARM>(a, T, ch);
      else search_body_coop<N, K, L, WARM>(a, T, ch, sub, gmask);
    }
  }
}

template <int N, int K>
__global__ void __launch_bounds__(128) screen_persist(const MixedArgs a, int set) {
  const DevMixed& T = a.tab[set];
  const unsigned total = a.list_identity ? unsigned(a.n) : a.ws_sched[SCHED_COUNT + set];
  const int* list = a.ws_list + int64_t(set) * MIXED_CHUNK;
  const int lane = threadIdx.x & 31;
  for (;;) {
    const unsigned base = steal(a.ws_sched + SCHED_STEAL + set * 6 + 5, 32u);
    if (base >= total) break;
    const unsigned i = base + unsigned(lane);
    if (i < total) screen_body<N, K>(a, T, a.list_identity ? int64_t(i) : int64_t(list[i]), a.ws_sched + SCHED_FIXQ + set);
  }
}

template <int N, int K>
__global__ void __launch_bounds__(128) fix_persist(const MixedArgs a, int set, int rounds) {
  const DevMixed& T = a.tab[set];
  const unsigned total = a.ws_sched[SCHED_FIXQ + set];
  const int lane = threadIdx.x & 31;
  for (;;) {
    const unsigned base = steal(a.ws_sched + SCHED_STEAL + set * 6 + 2, 32u);
    if (base >= total) break;
    const unsigned i = base + unsigned(lane);
    if (i < total) fix_body<N, K>(a, T, unsigned(a.ws_fixq[i]), rounds);
  }
}

// The second judge pass over the channels the fix changed.
template <int N, int K, bool DF>
__global__ void __launch_bounds__(128, DF ? 4 : 6) judge_fixed_persist(const __grid_constant__ MixedArgs a,
    const __grid_constant__ DevMixed T, int set) {
  const unsigned total = a.ws_sched[SCHED_FIXQ + set];
  const int lane = threadIdx.x & 31;
  for (;;) {
    const unsigned base = steal(a.ws_sched + SCHED_STEAL + set * 6 + 1, 32u);
    if (base >= total) break;
    const unsigned i = base + unsigned(lane);
    if (i < total) {
      const int64_t ch = int64_t(unsigned(a.ws_fixq[i]));
      if constexpr (DF) judge_df_body<N, K>(a, T, ch, a.ws_sched + SCHED_QUEUE + set, nullptr);
      else judge_body<N, K>(a, a.tab[set], ch, a.ws_sched + SCHED_QUEUE + set, nullptr);
    }
  }
}

template <int N, int K, bool DF>
__global__ void __launch_bounds__(128, DF ? 4 : 6) judge_persist(const __grid_constant__ MixedArgs a,
    const __grid_constant__ DevMixed T, int set, int fixq) {
  const unsigned total = a.list_identity ? unsigned(a.n) : a.ws_sched[SCHED_COUNT + set];
  const int* list = a.ws_list + int64_t(set) * MIXED_CHUNK;
  const int lane = threadIdx.x & 31;
  for (;;) {
    const unsigned base = steal(a.ws_sched + SCHED_STEAL + set * 6 + 3, 32u);
    if (base >= total) break;
    const unsigned i = base + unsigned(lane);
    if (i < total) {
      const int64_t ch = a.list_identity ? int64_t(i) : int64_t(list[i]);
      unsigned* fix_count = fixq ? a.ws_sched + SCHED_FIXQ + set : nullptr;
      if constexpr (DF) judge_df_body<N, K>(a, T, ch, a.ws_sched + SCHED_QUEUE + set, fix_count);
      else judge_body<N, K>(a, a.tab[set], ch, a.ws_sched + SCHED_QUEUE + set, fix_count);
    }
  }
}

template <int N, int K>
__global__ void __launch_bounds__(128) repair_persist(const MixedArgs a, int set) {
  const DevMixed& T = a.tab[set];
  const unsigned total = a.ws_sched[SCHED_QUEUE + set];
  const int lane = threadIdx.x & 31;
  for (;;) {
    const unsigned base = steal(a.ws_sched + SCHED_STEAL + set * 6 + 4, 32u);
    if (base >= total) break;
    const unsigned i = base + unsigned(lane);
    if (i < total) judge_repair<N, K>(a, T, int64_t(a.ws_queue[i]));
  }
}

// Resident blocks per SM of a kernel at a block size, from the occupancy
// calculator, cached per (kernel, block size).
int resident_blocks(const void* fn, int block) {
  static std::mutex mu;
  static const void* fns[64];
  static int blocks[64], occ[64], used = 0;
  std::lock_guard<std::mutex> g(mu);
  for (int i = 0; i < used; ++i)
    if (fns[i] == fn && blocks[i] == block) return occ[i];
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, 0) != cudaSuccess || n < 1) n = 1;
  if (used < 64) {
    fns[used] = fn;
    blocks[used] = block;
    occ[used++] = n;
  }
  return n;
}

// One wave of a persistent kernel: resident blocks per SM (capped by
// blocks_per_sm when set) times the SMs.
template <typename Kern>
unsigned wave(Kern* fn, int block, const MixedArgs& a) {
  int per_sm = resident_blocks(reinterpret_cast<const void*>(fn), block);
  if (a.blocks_per_sm > 0 && a.blocks_per_sm < per_sm) per_sm = a.blocks_per_sm;
  return unsigned(per_sm * (a.sms > 0 ? a.sms : 1));
}

template <int N, int K, int L, bool WARM>
cudaError_t launch_search(const MixedArgs& a, int set, int block, cudaStream_t s) {
  search_persist<N, K, L, WARM><<<wave(search_persist<N, K, L, WARM>, block, a), block, 0, s>>>(a, set);
  return cudaGetLastError();
}

template <int N, int K, bool WARM>
cudaError_t launch_set(const MixedArgs& a, int set, int block, int lanes, cudaStream_t s, LaunchTimer* tm) {
  if (tm) tm->mark(MF_K_SEARCH, s);
  cudaError_t e = cudaErrorInvalidValue;
  switch (lanes) {
    // lanes per channel = 32 / channels per warp (32, 8, 4, 2, 1)
    case 1: e = launch_search<N, K, 1, WARM>(a, set, block, s); break;
    case 4: e = launch_search<N, K, 4, WARM>(a, set, block, s); break;
    case 8: e = launch_search<N, K, 8, WARM>(a, set, block, s); break;
    case 16: e = launch_search<N, K, 16, WARM>(a, set, block, s); break;
    case 32: e = launch_search<N, K, 32, WARM>(a, set, block, s); break;
    default: break;
  }
  if (e != cudaSuccess) return e;
  // cold starts screen before the judge; warm starts let the judge queue the
  // few channels that need a column and judge them again after the fix
  if (!WARM) {
    if (tm) tm->mark(MF_K_SCREEN, s);
    screen_persist<N, K><<<wave(screen_persist<N, K>, 128, a), 128, 0, s>>>(a, set);
    if (tm) tm->mark(MF_K_FIX, s);
    fix_persist<N, K><<<wave(fix_persist<N, K>, 128, a), 128, 0, s>>>(a, set, 2);
  }
  if (tm) tm->mark(MF_K_JUDGE, s);
  if (a.judge_df) judge_persist<N, K, true><<<wave(judge_persist<N, K, true>, 128, a), 128, 0, s>>>(a, a.tab[set], set, WARM);
  else judge_persist<N, K, false><<<wave(judge_persist<N, K, false>, 128, a), 128, 0, s>>>(a, a.tab[set], set, WARM);
  if (WARM) {
    if (tm) tm->mark(MF_K_FIX, s);
    fix_persist<N, K><<<wave(fix_persist<N, K>, 128, a), 128, 0, s>>>(a, set, 1);
    if (tm) tm->mark(MF_K_REJUDGE, s);
    if (a.judge_df)
      judge_fixed_persist<N, K, true><<<wave(judge_fixed_persist<N, K, true>, 128, a), 128, 0, s>>>(a, a.tab[set], set);
    else
      judge_fixed_persist<N, K, false><<<wave(judge_fixed_persist<N, K, false>, 128, a), 128, 0, s>>>(a, a.tab[set], set);
  }
  if (tm) tm->mark(MF_K_REPAIR, s);
  repair_persist<N, K><<<wave(repair_persist<N, K>, 128, a), 128, 0, s>>>(a, set);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fit_mixed_persistent(const MixedArgs& a, int block, int lanes, cudaStream_t s, LaunchTimer* tm) {
  if (a.n == 0) return cudaSuccess;
  if (block <= 0) block = 128;
  if (block % 32 || block > 512 || !a.ws_list || !a.ws_sched) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(a.ws_sched, 0, sizeof(unsigned) * SCHED_WORDS, s);
  if (e != cudaSuccess) return e;
  if (!a.list_identity) {
    if (tm) tm->mark(MF_K_PARTITION, s);
    partition_kernel<<<wave(partition_kernel, 256, a), 256, 0, s>>>(a);
    e = cudaGetLastError();
  }
  for (int t = 0; t < a.n_ctypes && e == cudaSuccess; ++t) {
    const DevMixed& T = a.tab[t];
    const bool warm = a.warm_mask && t == a.warm_set;
    if (T.N == 10 && T.K == 10) {
      e = warm ? launch_set<10, 10, true>(a, t, block, lanes, s, tm) : launch_set<10, 10, false>(a, t, block, lanes, s, tm);
    } else if (T.N == 8 && T.K == 8 && !warm) {
      e = launch_set<8, 8, false>(a, t, block, lanes, s, tm);
    } else {
      e = cudaErrorInvalidValue;
    }
  }
  return e;
}

}  // namespace mfgb
