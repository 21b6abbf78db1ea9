// Batch work queue: one persistent launch advances many complex64 solves of
// different grid sizes by `steps` full steps.
//
// The work of the launch is a list of items in one global order: for every
// pass of every sub-step of every step (a phase: column pass, row pass,
// column pass, ...), for every solve, the pass's tiles (column items: COLS
// columns of one component) or line groups (row items: ROWS rows of both
// components).  Blocks claim items from a device counter in that order.  An
// item of phase q of solve s needs every item of phase q - 1 of the same
// solve (a 2-D transform needs all lines of the previous pass); the
// counter of finished items of that phase is waited on before the item
// runs.  Every item an item waits on comes earlier in the order, so it was
// claimed by a block that is resident (the launch is cooperative: every
// block is resident) and is either finished or running; the earliest
// unfinished item never waits, so the launch always progresses.  The wait
// is bounded all the same (1 s of %globaltimer or 2^26 polls): a wait that
// gives up sets the error word and the abort flag, and every block stops
// claiming.
//
// An item runs the same pass code as the single-solve kernels (row_body /
// col_body), with the item's position instead of the block's, plain loads
// and stores of the state (no bulk copies: the state was written by other
// blocks of this launch), in fixed 512-thread shapes per line length.
// Blocks claim SGPE_QUEUE_CHUNK consecutive items at a time.  Producers
// publish finished items with a block barrier followed by one thread's
// device-scope release reduction on the phase's counter; consumers read the
// counter with device-scope acquire loads, then pass a block barrier, after
// which the block's plain loads see the producers' stores.
#pragma once
#include "sgpe_kernels.cuh"

namespace sgpe {

// Threads of a block (= of an item) and resident blocks per SM requested
// from the compiler (register cap).
#ifndef SGPE_QUEUE_THREADS
#define SGPE_QUEUE_THREADS 512
#endif
#ifndef SGPE_QUEUE_MINB
#define SGPE_QUEUE_MINB 2
#endif
constexpr int kQueueThreads = SGPE_QUEUE_THREADS;
// Items claimed at once: consecutive items of one solve's pass run in one
// call of the item body, so that the call's register saves and the claim
// are paid once for all of them.
#ifndef SGPE_QUEUE_CHUNK
#define SGPE_QUEUE_CHUNK 8
#endif
constexpr unsigned kQueueChunk = SGPE_QUEUE_CHUNK;
constexpr int kQueueClasses = 7;
enum { kErrQueueWait = 2 };

// Line lengths of the queue kernel (size classes).
__host__ __device__ constexpr int queue_size(int c) {
  return c == 0 ? 128 : c == 1 ? 192 : c == 2 ? 256 : c == 3 ? 384 : c == 4 ? 512 : c == 5 ? 768 : 1024;
}
inline int queue_class(int n) {
  for (int c = 0; c < kQueueClasses; ++c)
    if (queue_size(c) == n) return c;
  return -1;
}

// Item shapes: E points per thread (16 for powers of two, 12 for 3 * 2^k,
// within the 64 registers of two 512-thread blocks per SM); a row item is
// ROWS rows of both components, a column item COLS columns of one.
template <int N> struct QueueShape {
  static constexpr int E = (N % 3 == 0) ? 12 : 16;
  static constexpr int T = N / E;
  static constexpr int ROWS = kQueueThreads / (2 * T);
  static constexpr int COLS = kQueueThreads / T;
  static constexpr size_t ROW_SMEM = 2ull * ROWS * (N + N / E) * sizeof(float2);
  static constexpr size_t COL_SMEM = size_t(COLS) * (N + N / E + 2) * sizeof(float2);
  static_assert(ROWS >= 1 && COLS >= 1 && 2 * T * ROWS == kQueueThreads && T * COLS == kQueueThreads,
                "queue items fill the block");
};

// The same shapes for a line length known at run time (host side).
__host__ __device__ constexpr int queue_e(int n) { return (n % 3 == 0) ? 12 : 16; }
__host__ __device__ constexpr int queue_rows(int n) { return kQueueThreads / (2 * (n / queue_e(n))); }
__host__ __device__ constexpr int queue_cols(int n) { return kQueueThreads / (n / queue_e(n)); }

struct QueueSolve {
  const ColArgs<float>* col;  // column pass after sub-step (0 -> 0), (0 -> 1), (1 -> 0)
  const RowArgs<float>* row;  // row pass of sub-steps 0, 1
  int cls_x, cls_y;           // size classes of nx (row lines) and ny (column lines)
  int col_tiles;              // column items per component: nx / COLS(ny)
  int row_items;              // ny / ROWS(nx)
};

struct QueueArgs {
  const QueueSolve* solves;
  const int* col_first;  // [n + 1] first column item of each solve in a column phase
  const int* row_first;  // [n + 1] first row item of each solve in a row phase
  int n;                 // solves
  int phases;            // 6 * steps
  unsigned* claim;       // next item to claim
  unsigned* done;        // [n][phases] finished items
  int* err;              // device error word (kErrQueueWait when a wait gave up)
  int* abort;            // set with err: blocks stop claiming
};

// Publish one finished item: a release reduction by the thread that
// follows the block barrier covers the whole block's stores.
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Wait until *p >= need; false when the abort flag is set or the limit
// (1 s or 2^26 polls) is reached.
__device__ __forceinline__ bool queue_wait(const unsigned* p, unsigned need, const int* abort) {
  if (ld_acquire(p) >= need) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned i = 0; i < (1u << 26); ++i) {
    __nanosleep(32);
    if (ld_acquire(p) >= need) return true;
    if ((i & 255) == 255) {
      if (*reinterpret_cast<const volatile int*>(abort) != 0) return false;
      if (global_ns() - t0 > 1000000000ull) return false;
    }
  }
  return false;
}

// Each item body is its own function, so that it gets its own register
// allocation (one inlined kernel over all line lengths spills); a call runs
// `count` consecutive items of one solve's pass, from item `first`.
template <int N>
__device__ __noinline__ void queue_col(const ColArgs<float>& a, int first, int count, int tiles) {
  using S = QueueShape<N>;
  for (int t = first; t < first + count; ++t) {
    if (t > first) __syncthreads();
    col_body<float, N, S::E, S::COLS, false, true>(a, BlockPos{t % tiles, t / tiles, tiles});
  }
}
template <int N>
__device__ __noinline__ void queue_row(const RowArgs<float>& a, int first, int count, int items) {
  using S = QueueShape<N>;
  for (int t = first; t < first + count; ++t) {
    if (t > first) __syncthreads();
    row_body<float, N, S::E, S::ROWS, true, false, true>(a, BlockPos{t, 0, items});
  }
}

__device__ __forceinline__ int find_solve(const int* first, int n, int idx) {
  int lo = 0, hi = n;  // first[lo] <= idx < first[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(first + mid) <= idx) lo = mid;
    else hi = mid;
  }
  return lo;
}

// The kernels are compiled in sgpe_queue_f32.cu only.
#ifdef SGPE_QUEUE_KERNELS
__global__ void __launch_bounds__(kQueueThreads, SGPE_QUEUE_MINB) batch_queue_kernel(const QueueArgs q) {
  __shared__ unsigned s_item;
  __shared__ int s_stop;
  const int tid = threadIdx.x;
  const unsigned ncol = unsigned(__ldg(q.col_first + q.n));
  const unsigned nrow = unsigned(__ldg(q.row_first + q.n));
  const unsigned period = ncol + nrow;  // items of one column and one row phase
  const unsigned total = period * unsigned(q.phases / 2);
  // thread 0 claims the next chunk while the block runs the current one
  if (tid == 0) s_item = atomicAdd(q.claim, kQueueChunk);
  __syncthreads();
  for (;;) {
    const unsigned first = s_item;
    if (first >= total) return;
    const unsigned end = min(first + kQueueChunk, total);
    unsigned next = 0;
    // the chunk's items, one run of consecutive items of one solve's pass
    // at a time (a chunk may cross into the next solve or pass)
    for (unsigned it = first; it < end;) {
      const unsigned pair = it / period;  // step * 3 + sub-step
      const unsigned rem = it - pair * period;
      const bool col = rem < ncol;
      const int phase = int(2 * pair + (col ? 0 : 1));
      const int idx = int(col ? rem : rem - ncol);
      const int s = find_solve(col ? q.col_first : q.row_first, q.n, idx);
      const int b = idx - __ldg((col ? q.col_first : q.row_first) + s);
      const QueueSolve& sv = q.solves[s];
      const int n_items = col ? 2 * sv.col_tiles : sv.row_items;
      const int run = min(int(end - it), n_items - b);
      if (tid == 0) {
        bool ok = *reinterpret_cast<volatile int*>(q.abort) == 0;
        if (ok && phase > 0) {
          const int need = (phase & 1) ? 2 * sv.col_tiles : sv.row_items;  // items of phase - 1
          ok = queue_wait(q.done + (long long)s * q.phases + phase - 1, unsigned(need), q.abort);
          if (!ok) {
            atomicExch(q.err, kErrQueueWait);
            atomicExch(q.abort, 1);
          }
        }
        s_stop = ok ? 0 : 1;
        if (ok && it == first) next = atomicAdd(q.claim, kQueueChunk);  // used after this chunk
      }
      __syncthreads();  // every thread has read s_item and s_stop is set
      if (s_stop) return;
      const int sub = int(pair % 3u);
      if (col) {
        const ColArgs<float>& a = sv.col[sub];
        switch (sv.cls_y) {
          case 0: queue_col<128>(a, b, run, sv.col_tiles); break;
          case 1: queue_col<192>(a, b, run, sv.col_tiles); break;
          case 2: queue_col<256>(a, b, run, sv.col_tiles); break;
          case 3: queue_col<384>(a, b, run, sv.col_tiles); break;
          case 4: queue_col<512>(a, b, run, sv.col_tiles); break;
          case 5: queue_col<768>(a, b, run, sv.col_tiles); break;
          default: queue_col<1024>(a, b, run, sv.col_tiles); break;
        }
      } else {
        const RowArgs<float>& a = sv.row[sub == 1 ? 1 : 0];
        switch (sv.cls_x) {
          case 0: queue_row<128>(a, b, run, sv.row_items); break;
          case 1: queue_row<192>(a, b, run, sv.row_items); break;
          case 2: queue_row<256>(a, b, run, sv.row_items); break;
          case 3: queue_row<384>(a, b, run, sv.row_items); break;
          case 4: queue_row<512>(a, b, run, sv.row_items); break;
          case 5: queue_row<768>(a, b, run, sv.row_items); break;
          default: queue_row<1024>(a, b, run, sv.row_items); break;
        }
      }
      __syncthreads();  // every thread's stores of the run are done
      if (tid == 0) red_release_add(q.done + (long long)s * q.phases + phase, unsigned(run));
      it += unsigned(run);
    }
    if (tid == 0) s_item = next;
    __syncthreads();
  }
}

// Check of the queue's bounded wait: one block waits for a counter that
// nothing increments; records whether the wait ended by its limit and how
// long it took.
__global__ void queue_wait_check_kernel(const unsigned* never, const int* no_abort, int* gave_up,
                                        unsigned long long* waited_ns) {
  if (threadIdx.x == 0) {
    const unsigned long long t0 = global_ns();
    const bool ok = queue_wait(never, 1u, no_abort);
    *gave_up = ok ? 0 : 1;
    *waited_ns = global_ns() - t0;
  }
}

#endif  // SGPE_QUEUE_KERNELS

// Host side (sgpe_queue_f32.cu).
size_t queue_smem_bytes();
int queue_resident_blocks();  // blocks of the queue kernel that fit on the current device at once
cudaError_t launch_batch_queue(const QueueArgs& q, int grid, cudaStream_t s);
cudaError_t check_queue_wait(int* gave_up, double* waited_ms);

}  // namespace sgpe
