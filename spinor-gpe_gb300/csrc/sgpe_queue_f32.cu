// Batch work queue kernel (complex64): host-side launch helpers.
#define SGPE_QUEUE_KERNELS
#include "sgpe_queue.cuh"

namespace sgpe {

namespace {
template <int N> constexpr size_t class_smem() {
  return QueueShape<N>::ROW_SMEM > QueueShape<N>::COL_SMEM ? QueueShape<N>::ROW_SMEM : QueueShape<N>::COL_SMEM;
}
constexpr size_t cmax_sz(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kQueueSmem =
    cmax_sz(cmax_sz(cmax_sz(class_smem<128>(), class_smem<192>()), cmax_sz(class_smem<256>(), class_smem<384>())),
            cmax_sz(cmax_sz(class_smem<512>(), class_smem<768>()), class_smem<1024>()));

cudaError_t queue_smem_attr() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static unsigned long long done = 0;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(batch_queue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kQueueSmem));
  if (e == cudaSuccess) done |= bit;
  return e;
}
}  // namespace

size_t queue_smem_bytes() { return kQueueSmem; }

int queue_resident_blocks() {
  if (queue_smem_attr() != cudaSuccess) return 0;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_queue_kernel, kQueueThreads, kQueueSmem) !=
      cudaSuccess)
    return 0;
  return per_sm * sms;
}

// A cooperative launch: every block of the grid is resident at once, which
// the queue's waits between items rely on (the grid must not exceed
// queue_resident_blocks()).
cudaError_t launch_batch_queue(const QueueArgs& q, int grid, cudaStream_t s) {
  cudaError_t e = queue_smem_attr();
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kQueueThreads);
  cfg.dynamicSmemBytes = kQueueSmem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, batch_queue_kernel, q);
}

cudaError_t check_queue_wait(int* gave_up, double* waited_ms) {
  unsigned* never = nullptr;
  int* ints = nullptr;
  unsigned long long* ns = nullptr;
  cudaError_t e = cudaMalloc(&never, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&ints, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&ns, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(never, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(ints, 0, 2 * sizeof(int));
  if (e == cudaSuccess) {
    queue_wait_check_kernel<<<1, 32>>>(never, ints, ints + 1, ns);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int g = 0;
  unsigned long long t = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&g, ints + 1, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&t, ns, sizeof(t), cudaMemcpyDeviceToHost);
  if (never) cudaFree(never);
  if (ints) cudaFree(ints);
  if (ns) cudaFree(ns);
  if (e == cudaSuccess) {
    *gave_up = g;
    *waited_ms = double(t) * 1e-6;
  }
  return e;
}

}  // namespace sgpe
