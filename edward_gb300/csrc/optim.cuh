// Element-wise optimizer updates in TensorFlow's formulation
// (tf.train.*Optimizer apply_dense), used by the fused step kernels whose
// parameters live in one flat buffer.  Slots s0 / s1 hold the optimizer's
// accumulators; b1p / b2p are Adam's running beta powers before this step.
#pragma once

#include "edg_common.cuh"

namespace edg {

__device__ __forceinline__ float opt_lr(const edg_opt_t& o, int64_t step) {
  if (o.decay_steps <= 0) return o.lr0;
  float p = (float)step / (float)o.decay_steps;
  if (o.staircase) p = floorf(p);
  return o.lr0 * powf(o.decay_rate, p);
}

__device__ __forceinline__ float opt_apply(const edg_opt_t& o, float p, float g, float* s0,
                                           float* s1, float lr, float b1p, float b2p) {
  switch (o.optimizer) {
    case EDG_OPT_ADAM: {
      const float lr_t = lr * sqrtf(1.0f - b2p) / (1.0f - b1p);
      const float m = o.beta1 * *s0 + (1.0f - o.beta1) * g;
      const float v = o.beta2 * *s1 + (1.0f - o.beta2) * g * g;
      *s0 = m;
      *s1 = v;
      return p - lr_t * m / (sqrtf(v) + o.epsilon);
    }
    case EDG_OPT_SGD:
      return p - lr * g;
    case EDG_OPT_MOMENTUM: {
      const float acc = o.momentum * *s0 + g;
      *s0 = acc;
      return p - lr * acc;
    }
    case EDG_OPT_ADAGRAD: {
      const float acc = *s0 + g * g;
      *s0 = acc;
      return p - lr * g * rsqrtf(acc);
    }
    case EDG_OPT_RMSPROP: {
      const float ms = o.rho * *s0 + (1.0f - o.rho) * g * g;
      const float mom = o.momentum * *s1 + lr * g / sqrtf(ms + o.epsilon);
      *s0 = ms;
      *s1 = mom;
      return p - mom;
    }
    default: {  // EDG_OPT_ADADELTA
      const float acc = o.rho * *s0 + (1.0f - o.rho) * g * g;
      const float upd = sqrtf(*s1 + o.epsilon) / sqrtf(acc + o.epsilon) * g;
      *s0 = acc;
      *s1 = o.rho * *s1 + (1.0f - o.rho) * upd * upd;
      return p - lr * upd;
    }
  }
}

}  // namespace edg
