// SIMT building block shared by the GLM kernels (csrc/glm.cu) and the ragged
// hierarchical HMC kernel (csrc/hier.cu): the log-likelihood and its adjoint
// of CT parameter vectors over a row range of X, streamed through shared
// memory.  See glm_grad_eval below.
#pragma once

#include "edg_common.cuh"

namespace edg {

constexpr int kThreads = 256;

// A tile is RT rows x CT vectors; each of the 256 threads computes RPT rows x
// 4 vectors of its eta (RPT = 2: 8 outputs per thread, the default; RPT = 1
// halves the rows per tile for problems whose row count spreads over too few
// blocks otherwise).
template <int CT, int RPT = 2>
struct Tile {
  static_assert(CT == 8 || CT == 16 || CT == 32, "chains per block must be 8, 16 or 32");
  static_assert(RPT == 1 || RPT == 2, "rows per thread must be 1 or 2");
  static constexpr int RT = 1024 * RPT / CT;  // rows per tile
  static constexpr int CQ = CT / 4;           // chain quads
};

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, int src_bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Shared-memory views used by glm_grad_eval.
struct GradSmem {
  float* Xs;      // [2][RT][PP]  X tiles (bias column = 1, padding = 0)
  float* ys;      // [2][RT]
  float* Rs;      // [RT][CT]     residuals of the current tile
  float* Zt;      // [PP][CT]     parameter vectors, transposed
  float* G;       // [CT][PP]     OUT: likelihood gradient (scaled)
  float* Gpart;   // [4096]       row-group partials of G
  double* llred;  // [RT/RPT][CT] per-thread log-lik partials
  double* ll;     // [CT]         OUT: log-likelihood (scaled)
};

template <int CT, int RPT = 2>
__host__ __device__ constexpr size_t grad_smem_floats(int PP) {
  return (size_t)2 * Tile<CT, RPT>::RT * PP + 2 * Tile<CT, RPT>::RT +
         (size_t)Tile<CT, RPT>::RT * CT + (size_t)PP * CT + (size_t)CT * PP + 4096;
}
template <int CT, int RPT = 2>
__host__ __device__ constexpr size_t grad_smem_doubles() {
  return (size_t)(Tile<CT, RPT>::RT / RPT) * CT + CT;
}

// Carves GradSmem from `base` (16-byte aligned); returns the first free byte.
template <int CT, int RPT = 2>
__device__ unsigned char* carve_grad(unsigned char* base, int PP, GradSmem& S) {
  constexpr int RT = Tile<CT, RPT>::RT;
  double* d = reinterpret_cast<double*>(base);
  S.llred = d;
  d += (RT / RPT) * CT;
  S.ll = d;
  d += CT;
  float* f = reinterpret_cast<float*>(d);
  S.Xs = f;
  f += 2 * RT * PP;
  S.Rs = f;
  f += RT * CT;
  S.Zt = f;
  f += PP * CT;
  S.G = f;
  f += CT * PP;
  S.Gpart = f;
  f += 4096;
  S.ys = f;
  f += 2 * RT;
  return reinterpret_cast<unsigned char*>(f);
}

// Constant columns of both X buffers: bias column = 1 (if any), padding = 0.
template <int CT, int RPT = 2>
__device__ void init_x_pad(const GLMDev& m, const GradSmem& S) {
  constexpr int RT = Tile<CT, RPT>::RT;
  const int extra = m.PP - m.D;
  for (int i = threadIdx.x; i < 2 * RT * extra; i += kThreads) {
    const int row = i / extra, col = m.D + i % extra;
    S.Xs[row * m.PP + col] = (m.bias && col == m.D) ? 1.0f : 0.0f;
  }
}

template <int CT, int RPT = 2>
__device__ __forceinline__ void issue_tile(const GLMDev& m, float* Xdst, float* ydst, int row0,
                                           int row_end) {
  constexpr int RT = Tile<CT, RPT>::RT;
  const int nrows = min(RT, row_end - row0);
  const int D = m.D, PP = m.PP;
  const int total = RT * D;
  const float* Xsrc = m.X + (size_t)row0 * D;
  const int valid = nrows * D;
  // incremental (r, d) walk: e = tid + k * kThreads
  int r = threadIdx.x / D, d = threadIdx.x - (threadIdx.x / D) * D;
  const int step_r = kThreads / D, step_d = kThreads - (kThreads / D) * D;
  for (int e = threadIdx.x; e < total; e += kThreads) {
    const bool ok = e < valid;
    cp_async4(Xdst + r * PP + d, ok ? (const void*)(Xsrc + e) : (const void*)m.X, ok ? 4 : 0);
    r += step_r;
    d += step_d;
    if (d >= D) {
      d -= D;
      ++r;
    }
  }
  for (int i = threadIdx.x; i < RT; i += kThreads) {
    const bool ok = i < nrows;
    cp_async4(ydst + i, ok ? (const void*)(m.y + row0 + i) : (const void*)m.y, ok ? 4 : 0);
  }
}

// Log-likelihood term and residual d/d eta for one (row, vector).  Bernoulli:
// e = e^-|eta| = 2^(-|eta| log2 e) <= 1 and a = 1 + e give sigmoid(eta) = 1/a
// (eta >= 0) or e/a and log1p(e) = ln 2 * log2(a) (absolute error ~2e-7).
__device__ __forceinline__ void lik_term(const GLMDev& m, float y, float eta, float& ll,
                                         float& resid) {
  if (m.lik == EDG_LIK_BERNOULLI) {
    const float e = ex2_approx(-kLog2e * fabsf(eta));
    const float a = 1.0f + e;
    const float s = rcp_approx(a);
    ll = -(fmaxf(eta, 0.0f) - eta * y + kLn2 * lg2_approx(a));
    resid = y - (eta >= 0.0f ? s : e * s);
  } else {
    const float diff = y - eta;
    ll = -0.5f * diff * diff * m.inv_lik_var - m.lik_norm;
    resid = diff * m.inv_lik_var;
  }
}

// Log-likelihood (and gradient) of CT vectors S.Zt over rows [row_begin, row_end).
// All threads of the block must call it.  On return S.G / S.ll hold the
// results (multiplied by dscale) and a __syncthreads() has been done.
template <int CT, int RPT = 2>
__device__ void glm_grad_eval(const GLMDev& m, int row_begin, int row_end, const GradSmem& S,
                              bool need_ll, bool need_grad, float dscale,
                              bool first_issued = false) {
  constexpr int RT = Tile<CT, RPT>::RT, CQ = Tile<CT, RPT>::CQ;
  const int tid = threadIdx.x;
  const int PP = m.PP, P4 = PP / 4;
  // phase A: rows RPT rp .. RPT rp + RPT - 1; chains 4cq..4cq+3
  const int cq = tid % CQ, rp = tid / CQ;
  // phase B: units of (chain quad, feature quad)
  const int U = CQ * P4;
  int H, nu, unit0, unit1, hgrp;
  if (U <= kThreads) {
    H = kThreads / U;
    hgrp = tid / U;
    unit0 = tid % U;
    unit1 = -1;
    nu = tid < U * H ? 1 : 0;
  } else {
    H = 1;
    hgrp = 0;
    unit0 = tid;
    unit1 = tid + kThreads;
    nu = (unit0 < U) + (unit1 < U);
  }
  float accB[2][16];
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int i = 0; i < 16; ++i) accB[k][i] = 0.0f;
  Kahan kll[4];

  const int ntiles = (row_end - row_begin + RT - 1) / RT;
  // (first_issued: the caller already issued and committed the first tile
  // into buffer 0, so that its copy overlaps the caller's own set-up work)
  if (!first_issued) {
    if (ntiles > 0) issue_tile<CT, RPT>(m, S.Xs, S.ys, row_begin, row_end);
    cp_async_commit();
  }
  for (int it = 0; it < ntiles; ++it) {
    const int buf = it & 1;
    if (it + 1 < ntiles)
      issue_tile<CT, RPT>(m, S.Xs + (buf ^ 1) * RT * PP, S.ys + (buf ^ 1) * RT,
                          row_begin + (it + 1) * RT, row_end);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const float* Xb = S.Xs + buf * RT * PP;
    const float* yb = S.ys + buf * RT;
    const int r0 = row_begin + it * RT;

    // ---- phase A: eta = X z
    float acc[RPT][4];
#pragma unroll
    for (int i = 0; i < RPT; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    const float4* xr0 = reinterpret_cast<const float4*>(Xb + (RPT * rp) * PP);
    const float4* xr1 = reinterpret_cast<const float4*>(Xb + (RPT * rp + RPT - 1) * PP);
    const float4* zt = reinterpret_cast<const float4*>(S.Zt);
    // (unrolled so that the next feature quad's loads issue before this
    // quad's FMAs; likewise the row loop of phase B below)
#pragma unroll 2
    for (int dq = 0; dq < P4; ++dq) {
      const float4 x0 = xr0[dq], x1 = xr1[dq];
      const float4 z0 = zt[(4 * dq + 0) * CQ + cq];
      const float4 z1 = zt[(4 * dq + 1) * CQ + cq];
      const float4 z2 = zt[(4 * dq + 2) * CQ + cq];
      const float4 z3 = zt[(4 * dq + 3) * CQ + cq];
#define EDG_ROWFMA(A, XV)                                                  \
  A[0] = fmaf(XV.x, z0.x, A[0]); A[1] = fmaf(XV.x, z0.y, A[1]);            \
  A[2] = fmaf(XV.x, z0.z, A[2]); A[3] = fmaf(XV.x, z0.w, A[3]);            \
  A[0] = fmaf(XV.y, z1.x, A[0]); A[1] = fmaf(XV.y, z1.y, A[1]);            \
  A[2] = fmaf(XV.y, z1.z, A[2]); A[3] = fmaf(XV.y, z1.w, A[3]);            \
  A[0] = fmaf(XV.z, z2.x, A[0]); A[1] = fmaf(XV.z, z2.y, A[1]);            \
  A[2] = fmaf(XV.z, z2.z, A[2]); A[3] = fmaf(XV.z, z2.w, A[3]);            \
  A[0] = fmaf(XV.w, z3.x, A[0]); A[1] = fmaf(XV.w, z3.y, A[1]);            \
  A[2] = fmaf(XV.w, z3.z, A[2]); A[3] = fmaf(XV.w, z3.w, A[3]);
      EDG_ROWFMA(acc[0], x0)
      if (RPT == 2) {
        EDG_ROWFMA(acc[RPT - 1], x1)
      }
#undef EDG_ROWFMA
    }
    // ---- epilogue: residuals and log-lik terms
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int lr = RPT * rp + i;
      const bool valid = r0 + lr < row_end;
      const float yv = yb[lr];
      float res[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float ll, rs;
        lik_term(m, yv, acc[i][j], ll, rs);
        res[j] = valid ? rs * dscale : 0.0f;
        if (need_ll && valid) kll[j].add(ll);
      }
      reinterpret_cast<float4*>(S.Rs + lr * CT)[cq] = make_float4(res[0], res[1], res[2], res[3]);
    }
    __syncthreads();
    // ---- phase B: G += resid^T X
    if (need_grad) {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int u = k == 0 ? unit0 : unit1;
        if (k >= nu) break;
        const int cqb = u % CQ, dqb = u / CQ;
        float* a = accB[k];
#pragma unroll 4
        for (int r = hgrp; r < RT; r += H) {
          const float4 rr = reinterpret_cast<const float4*>(S.Rs + r * CT)[cqb];
          const float4 xx = reinterpret_cast<const float4*>(Xb + r * PP)[dqb];
          const float rv[4] = {rr.x, rr.y, rr.z, rr.w};
          const float xv[4] = {xx.x, xx.y, xx.z, xx.w};
#pragma unroll
          for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int dd = 0; dd < 4; ++dd) a[c * 4 + dd] = fmaf(rv[c], xv[dd], a[c * 4 + dd]);
        }
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();

  // ---- combine row groups of G
  if (need_grad) {
    float* dst = (U <= kThreads) ? S.Gpart + hgrp * CT * PP : S.G;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (k >= nu) break;
      const int u = k == 0 ? unit0 : unit1;
      const int cqb = u % CQ, dqb = u / CQ;
#pragma unroll
      for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int dd = 0; dd < 4; ++dd)
          dst[(4 * cqb + c) * PP + 4 * dqb + dd] = accB[k][c * 4 + dd];
    }
    __syncthreads();
    if (U <= kThreads) {
      for (int idx = tid; idx < CT * PP; idx += kThreads) {
        float s = 0.0f;
        for (int h = 0; h < H; ++h) s += S.Gpart[h * CT * PP + idx];
        S.G[idx] = s;
      }
    }
  }
  // ---- FP64 reduction of the log-lik partials: one warp per vector, lanes
  // over the RT / 2 row-pair partials, then a fixed-order shuffle tree (GB300
  // runs FP64 at a small fraction of its FP32 rate, so a serial sum of RT / 2
  // terms by one thread per vector is slow)
  if (need_ll) {
#pragma unroll
    for (int j = 0; j < 4; ++j) S.llred[rp * CT + 4 * cq + j] = kll[j].value();
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    for (int c = warp; c < CT; c += kThreads / 32) {
      double s = 0.0;
      for (int q = lane; q < RT / RPT; q += 32) s += S.llred[q * CT + c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) S.ll[c] = s * (double)dscale;
    }
  }
  __syncthreads();
}

// Zt[d][c] = z[c][d] for a [CT][PP] block.
template <int CT>
__device__ __forceinline__ void transpose_into(const float* Z, float* Zt, int PP) {
  for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
    const int c = idx / PP, d = idx - c * PP;
    Zt[d * CT + c] = Z[idx];
  }
}

}  // namespace edg
