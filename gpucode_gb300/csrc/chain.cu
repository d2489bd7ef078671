/*
 * chain.cu -- step chaining on the device for the mixed-precision engine.
 *
 * The reference decides on the host, before every step, whether the
 * neighbour lists must be rebuilt (main.cpp:467-470: a device-to-host read of
 * the move flag each step).  A CUDA-graph conditional node keeps that
 * decision on the device but costs about 11 us per step on the GB300 even
 * when the rebuild does not run -- an eighth of a 200k-sphere step.  Here the
 * steps launch one another from the device instead (device graph launch):
 *
 *   step graph S[p] = [wall motion] -> [step kernel] -> [k_chain]
 *   rebuild graph R[p] = [k_clear_request] -> [the rebuild]
 *
 * Every kernel of S[p] first reads the rebuild request word (need): when it
 * is set they do nothing, and k_chain tail-launches R[p] and then S[p] again,
 * so the step runs on rebuilt lists.  Otherwise k_chain turns the step's move
 * flag into the request for the next step (flag > 0 -> need = 1, flag = 0)
 * and, while steps are left, tail-launches S[1-p].  A tail launch starts when
 * the launching graph has completed, and work queued on the stream after the
 * host's launch waits for the whole chain.  The single-step graphs (one
 * host launch per step) are the same without the countdown.  For a
 * one-step call the host launches a second, host-instantiated copy of S1[p]:
 * launched from the host, a graph instantiated for device launch starts ~5 us
 * later, and a kernel of the host copy tail-launches the device graphs all the
 * same (a chain of many steps started from that copy measured ~1.5 us per
 * step slower, so longer calls launch S[p] itself).
 *
 * need is written only by k_chain and k_clear_request (and by the host
 * between launches), never while a step kernel runs, so every block of a
 * step kernel reads the same value.  The last step of a chain leaves a raised
 * request for the next call, which rebuilds before its first step: the
 * reference's order, the rebuild at the start of the step after the flag.
 *
 * This unit is compiled with relocatable device code (device-side
 * cudaGraphLaunch needs the device runtime); the step kernel is not, so its
 * register allocation is unchanged.
 */
#include "engine.h"

namespace dem {
namespace {

/* a tail launch that fails ends the chain early: error bit 8, which
 * dem_sync reports */
__device__ void tail(cudaGraphExec_t g, int* err) {
  if (cudaGraphLaunch(g, cudaStreamGraphTailLaunch) != cudaSuccess) atomicOr(err, 8);
}

__global__ void k_chain(StepCtl* ctl, int* flag, int* need, int* err, int p, int single) {
  if (*need) {
    /* this step was skipped: rebuild, then the same step */
    tail(ctl->rebuild[p], err);
    tail(single ? ctl->single[p] : ctl->step[p], err);
    return;
  }
  if (*flag > 0) *need = 1;
  *flag = 0;
  if (single) return;
  /* the countdown always moves, so the chain ends after `left` steps */
  const int left = ctl->left - 1;
  ctl->left = left;
  if (left > 0) tail(ctl->step[1 - p], err);
}

__global__ void k_set_left(StepCtl* ctl, int n) { ctl->left = n; }

__global__ void k_clear_request(int* flag, int* need) {
  *flag = 0;
  *need = 0;
}

}  // namespace

dem_status chain_launch_tail(StepCtl* ctl, int* flag, int* need, int* err, int parity, bool single, cudaStream_t s) {
  k_chain<<<1, 1, 0, s>>>(ctl, flag, need, err, parity, single ? 1 : 0);
  return cuda_check(cudaGetLastError(), "step chain launch");
}

dem_status chain_set_left(StepCtl* ctl, int nsteps, cudaStream_t s) {
  k_set_left<<<1, 1, 0, s>>>(ctl, nsteps);
  return cuda_check(cudaGetLastError(), "step chain count");
}

dem_status chain_clear_request(int* flag, int* need, cudaStream_t s) {
  k_clear_request<<<1, 1, 0, s>>>(flag, need);
  return cuda_check(cudaGetLastError(), "rebuild request reset");
}

}  // namespace dem
