// probes.cu -- two measurements behind the choice of one CUDA graph of
// per-kernel launches per step over a persistent step kernel: what one
// kernel node of a graph costs when the kernel does nothing (the price of a
// launch that stands down, as most of a step's rebin and list-build launches
// do between list rebuilds), and what one grid-wide barrier costs inside a
// cooperative kernel with every resident CTA (what a persistent kernel
// would pay between the phases of a step instead).  No counterpart in the
// reference.
#include <cstdio>
#include <vector>

#include "sim.h"

using namespace cgapi;

namespace {

constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) empty_kernel(int *flag) {
  if (flag && blockIdx.x == 0 && threadIdx.x == 0 && *flag == 12345) *flag = 0;
}

// `rounds` grid-wide barriers: thread 0 of each CTA adds to the counter and
// waits until every CTA has arrived; every wait gives up after `limit`
// polls, records that in err and returns (the launch is cooperative, so all
// CTAs are resident and the waits end)
__global__ void __launch_bounds__(kProbeThreads) barrier_kernel(unsigned *count, int rounds,
                                                                 long long limit, int *err) {
  __shared__ int stop;  // thread 0's reading of err, the same for the whole CTA
  for (int r = 1; r <= rounds; r++) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(count, 1u);
      const unsigned target = (unsigned)r * gridDim.x;
      long long polls = 0;
      while (*(volatile unsigned *)count < target) {
        if (++polls > limit) {
          atomicExch(err, 1);
          break;
        }
      }
      __threadfence();
      stop = *(volatile int *)err;
    }
    __syncthreads();
    if (stop) return;
  }
}

}  // namespace

extern "C" int comdgb_graph_node_cost(int device, double *us_per_node) {
  if (!us_per_node) return set_err(COMDGB_ERR_ARG, "null argument");
  CK(cudaSetDevice(device));
  int sms = 1;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  const int nodes = 64, reps = 20;
  cudaGraph_t g;
  cudaGraphExec_t ge;
  cudaEvent_t e0, e1;
  int rc = 0;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = 1;
  // grids like the stood-down launches of a step: several CTAs per SM
  for (int i = 0; i < nodes && !rc; i++) empty_kernel<<<4 * sms, kProbeThreads, 0, st>>>(nullptr);
  if (!rc && cudaStreamEndCapture(st, &g) != cudaSuccess) rc = 1;
  if (!rc && cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) rc = 1;
  if (!rc) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaGraphLaunch(ge, st);  // warm
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; r++) cudaGraphLaunch(ge, st);
    cudaEventRecord(e1, st);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      rc = 1;
    *us_per_node = 1e3 * ms / (nodes * reps);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
  }
  cudaStreamDestroy(st);
  if (rc) return set_err(COMDGB_ERR_CUDA, "graph node probe failed: %s",
                         cudaGetErrorString(cudaGetLastError()));
  return 0;
}

extern "C" int comdgb_grid_barrier_cost(int device, double *us_per_barrier) {
  if (!us_per_barrier) return set_err(COMDGB_ERR_ARG, "null argument");
  CK(cudaSetDevice(device));
  int coop = 0, sms = 1, per_sm = 0;
  CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
  if (!coop) return set_err(COMDGB_ERR_UNSUPPORTED, "device has no cooperative launch");
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, barrier_kernel, kProbeThreads, 0));
  if (per_sm < 1) per_sm = 1;
  const int grid = sms * per_sm, rounds = 200;
  const long long limit = 1ll << 22;  // polls; far above a barrier's wait
  unsigned *count = nullptr;
  int *err = nullptr;
  CK(cudaMalloc(&count, sizeof(unsigned)));
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
    cudaFree(count);
    return set_err(COMDGB_ERR_NOMEM, "cudaMalloc failed");
  }
  int rc = 0;
  float best = 1e30f;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int rep = 0; rep < 3 && !rc; rep++) {
    cudaMemset(count, 0, sizeof(unsigned));
    cudaMemset(err, 0, sizeof(int));
    int rounds_arg = rounds;
    long long limit_arg = limit;
    void *args[] = {&count, &rounds_arg, &limit_arg, &err};
    cudaEventRecord(e0);
    if (cudaLaunchCooperativeKernel((void *)barrier_kernel, grid, kProbeThreads, args, 0,
                                    nullptr) != cudaSuccess)
      rc = 1;
    cudaEventRecord(e1);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      rc = 1;
    int h_err = 0;
    cudaMemcpy(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost);
    if (h_err) rc = 2;
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(count);
  cudaFree(err);
  if (rc == 2) return set_err(COMDGB_ERR_CUDA, "grid barrier probe: a wait ran out");
  if (rc) return set_err(COMDGB_ERR_CUDA, "grid barrier probe failed: %s",
                         cudaGetErrorString(cudaGetLastError()));
  *us_per_barrier = 1e3 * best / rounds;
  return 0;
}
