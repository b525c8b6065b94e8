// Learned per-level variant selector: a 9 x 32 x 32 x 3 FP32 MLP evaluated
// by one warp inside the per-level decide kernels, so choosing a level's
// kernels needs no host round trip.
//
// The reference has no counterpart: its GPU BFS runs one fixed top-down
// kernel per level (src/algorithm/gpu/bfs.cu:9-35).  Here a level of a
// traversal may run as
//   kVarPush   sparse push: the frontier queue's rows, top-down;
//   kVarPull   bitmap pull: unvisited vertices scan their in-edges;
//   kVarDense  dense push: top-down without a touched queue, folded by a
//              sweep over every vertex (batched bitset traversal only).
// The frontier a level produces does not depend on the variant, so the
// choice changes speed only.  The network predicts log2 of each variant's
// duration (microseconds) from nine frontier statistics and the level runs
// the variant with the smallest prediction among those the traversal
// offers, when that prediction beats the direction heuristic's choice by a
// margin; otherwise (and without weights) the heuristic's choice runs.
//
// Weight layout (row-major, kSelWeights floats):
//   W1[32][9], b1[32], W2[32][32], b2[32], W3[3][32], b3[3]
#pragma once

#include "dawn_device.cuh"

namespace dawn {

constexpr int kSelIn = 9, kSelHidden = 32, kSelOut = 3;
constexpr int kSelWeights = kSelHidden * kSelIn + kSelHidden + kSelHidden * kSelHidden + kSelHidden +
                            kSelOut * kSelHidden + kSelOut;
static_assert(kSelWeights == DAWN_SELECTOR_WEIGHTS, "weight count differs from the public header");
static_assert(kSelHidden == 32, "one lane per hidden unit");

enum : int { kVarPush = 0, kVarPull = 1, kVarDense = 2 };

// log2(1 + max(x, 0)) in single precision (FP64 is slow on this part, and a
// decide kernel is a single warp: latency is its whole cost).
__device__ __forceinline__ float lg1p(float x) { return log2f(1.0f + fmaxf(x, 0.0f)); }

// The nine inputs, for the level about to run:
//   frontier vertices, frontier out-edges and in-edges of unfinished
//   vertices (each log-scaled against its total), graph size, average
//   degree, level, the previous frontier, the frontier's average degree
//   and the number of sources sharing the traversal.
__device__ __forceinline__ void sel_features(float (&x)[kSelIn], float n, float m, float nf, float mf, float mu,
                                             float level, float prev_nf, float nsrc) {
  const float ln = lg1p(n), lm = lg1p(m);
  const float rln = 1.0f / ln, rlm = 1.0f / lm;
  x[0] = lg1p(nf) * rln;
  x[1] = lg1p(mf) * rlm;
  x[2] = lg1p(mu) * rlm;
  x[3] = ln * (1.0f / 32.0f);
  x[4] = lg1p(m / fmaxf(n, 1.0f)) * (1.0f / 8.0f);
  x[5] = lg1p(level) * (1.0f / 12.0f);
  x[6] = lg1p(prev_nf) * rln;
  x[7] = lg1p(mf / fmaxf(nf, 1.0f)) * (1.0f / 16.0f);
  x[8] = nsrc * (1.0f / 256.0f);
}

// Pulls the weights (kSelWeights floats, under 6 KB) into L1 at kernel
// start, overlapping the control-block reads that precede the network.
__device__ __forceinline__ void sel_prefetch(const float* w) {
  const int lane = lane_id();
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int off = (lane + 32 * k) * 32;  // one 128-byte line per lane and step
    if (off < kSelWeights) asm volatile("prefetch.global.L1 [%0];" ::"l"(w + off));
  }
}

// Runs on all 32 lanes with identical x; returns the same variant on every
// lane: the allowed output (bit c of `allowed`) with the smallest predicted
// log-duration.  Every weight load is issued before the first use (one
// memory round trip) and the layers exchange activations through shared
// memory, so a decision costs well under a microsecond.
__device__ __forceinline__ int sel_pick(const float* __restrict__ w, const float (&x)[kSelIn], unsigned allowed,
                                        int heuristic, float margin) {
  __shared__ float s_h1[kSelHidden], s_h2[kSelHidden], s_out[kSelOut];
  const int j = lane_id();
  const float* W1 = w;
  const float* b1 = W1 + kSelHidden * kSelIn;
  const float* W2 = b1 + kSelHidden;
  const float* b2 = W2 + kSelHidden * kSelHidden;
  const float* W3 = b2 + kSelHidden;
  const float* b3 = W3 + kSelOut * kSelHidden;
  float w1[kSelIn], w2[kSelHidden], w3[kSelHidden];
#pragma unroll
  for (int i = 0; i < kSelIn; i++) w1[i] = __ldg(W1 + j * kSelIn + i);
#pragma unroll
  for (int i = 0; i < kSelHidden; i++) w2[i] = __ldg(W2 + j * kSelHidden + i);
  const int c = j < kSelOut ? j : 0;  // lanes 0-2 each own one output row
#pragma unroll
  for (int i = 0; i < kSelHidden; i++) w3[i] = __ldg(W3 + c * kSelHidden + i);
  const float bias1 = __ldg(b1 + j), bias2 = __ldg(b2 + j), bias3 = __ldg(b3 + c);
  float h = bias1;
#pragma unroll
  for (int i = 0; i < kSelIn; i++) h = fmaf(w1[i], x[i], h);
  s_h1[j] = fmaxf(h, 0.0f);
  __syncwarp();
  float h2 = bias2;
#pragma unroll
  for (int i = 0; i < kSelHidden; i++) h2 = fmaf(w2[i], s_h1[i], h2);
  s_h2[j] = fmaxf(h2, 0.0f);
  __syncwarp();
  if (j < kSelOut) {
    float o = bias3;
#pragma unroll
    for (int i = 0; i < kSelHidden; i++) o = fmaf(w3[i], s_h2[i], o);
    s_out[j] = o;
  }
  __syncwarp();
  int best = -1;
  float best_v = 0.0f;
#pragma unroll
  for (int k = 0; k < kSelOut; k++) {
    const float o = s_out[k];
    if (((allowed >> k) & 1u) && (best < 0 || o < best_v)) {
      best = k;
      best_v = o;
    }
  }
  // The heuristic's choice stands unless the network predicts another
  // variant faster by more than `margin` (log2 units): near-ties follow the
  // heuristic.
  const bool take = best >= 0 && best != heuristic && best_v + margin < s_out[heuristic];
  __syncwarp();  // the buffers may be reused by the caller's next call
  return take ? best : heuristic;
}

}  // namespace dawn
