// FP64 fast multipole kernels for the Laplace double-layer residual; see
// fmm.hpp for the formulation.  Complex numbers are (re, im) double pairs.
//
// Scaled expansions for a box with centre z_B and side s_B:
//   multipole  phi(z) = sum_k  M_k s^k / (z - z_B)^(k+1)
//   local      phi(z) = sum_l  L_l ((z - z_B) / s)^l
// Translations (d = z_B - z_C for M2L, e = z_child - z_parent):
//   P2M  M_k = sum_j c_j ((z_j - z_B) / s_B)^k
//   M2M  M_l(P) = sum_{k<=l} M_k(C) C(l,k) (s_C/s_P)^k ((z_C - z_P)/s_P)^(l-k)
//   M2L  L_l(B) = (-1)^l (s_B/d)^l / d * sum_k C(k+l,l) M_k(C) (s_C/d)^k
//   L2L  L_m(C) = sum_{l>=m} L_l(P) C(l,m) (s_C/s_P)^m (e/s_P)^(l-m)
//   P2L  L_l(B) -= c_j / w (s_B / w)^l,       w = z_j - z_B
//   L2P  phi(z) = sum_l L_l ((z - z_B)/s_B)^l
//   M2P  phi(z) = (1/w) sum_k M_k (s_C / w)^k, w = z - z_C
#include <cuda_runtime.h>
#include <math_constants.h>

#include "common.cuh"
#include "fmm.hpp"

namespace rskel {

namespace {

constexpr int kFmmThreads = 128;
constexpr int kMaxRhs = 8;  // right-hand sides per pass (larger batches loop)

struct Cx {
  double re, im;
};
__device__ __forceinline__ Cx cmul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ Cx cadd(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ Cx cinv(Cx a) {
  const double d = rcp(a.re * a.re + a.im * a.im);
  return {a.re * d, -a.im * d};
}
__device__ __forceinline__ Cx cscale(Cx a, double s) { return {a.re * s, a.im * s}; }

struct FmmArgs {
  const double *cx, *cy, *side, *zx, *zy, *binom;
  const int *pstart, *pcount, *parent, *slot_pt;
  const int *v_off, *v_idx, *w_off, *w_idx, *x_off, *x_idx, *u_off, *u_idx;
  const int* boxes;
  int p, npts, nrhs;
  const double* charge;  // complex, 2 * (slot + npts * q)
  double* mpole;         // complex, 2 * (k + p * (q + nrhs * box))
  double* local;
};

__device__ __forceinline__ Cx ld_c(const double* a, size_t i) { return {a[2 * i], a[2 * i + 1]}; }
__device__ __forceinline__ void st_c(double* a, size_t i, Cx v) {
  a[2 * i] = v.re;
  a[2 * i + 1] = v.im;
}

// Complex charges c_j = -(w_j / 2pi) (n_x + i n_y) mu_j in slot order.
__global__ void charges_kernel(Geo<double> g, const int* slot_pt, int npts, const double* mu,
                               int nrhs, double* charge) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)npts * nrhs) return;
  const int s = (int)(e % npts), q = (int)(e / npts);
  const int pt = slot_pt[s];
  const double a = -g.w[pt] * (1.0 / (2.0 * CUDART_PI)) * mu[pt + (size_t)npts * q];
  charge[2 * e] = a * g.nx[pt];
  charge[2 * e + 1] = a * g.ny[pt];
}

// P2M for every leaf (points staged 64 at a time).
__global__ void __launch_bounds__(kFmmThreads) p2m_kernel(FmmArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = a.boxes[blockIdx.x];
  const int s0 = a.pstart[b], cnt = a.pcount[b], p = a.p;
  Cx* pw = reinterpret_cast<Cx*>(smem);  // 64 x p
  const double cx = a.cx[b], cy = a.cy[b], is = rcp(a.side[b]);
  constexpr int kPer = 4;  // (k, q) pairs per thread (p * nrhs <= 512)
  Cx acc[kPer];
#pragma unroll
  for (int t = 0; t < kPer; ++t) acc[t] = {0.0, 0.0};
  for (int j0 = 0; j0 < cnt; j0 += 64) {
    const int jc = cnt - j0 < 64 ? cnt - j0 : 64;
    __syncthreads();
    for (int j = threadIdx.x; j < jc; j += blockDim.x) {
      const Cx rho = {(a.zx[s0 + j0 + j] - cx) * is, (a.zy[s0 + j0 + j] - cy) * is};
      Cx v = {1.0, 0.0};
      for (int k = 0; k < p; ++k) {
        pw[j * p + k] = v;
        v = cmul(v, rho);
      }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int e = threadIdx.x + t * blockDim.x;
      if (e >= p * a.nrhs) break;
      const int k = e % p, q = e / p;
      for (int j = 0; j < jc; ++j)
        acc[t] = cadd(acc[t], cmul(ld_c(a.charge, s0 + j0 + j + (size_t)a.npts * q), pw[j * p + k]));
    }
  }
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int e = threadIdx.x + t * blockDim.x;
    if (e >= p * a.nrhs) break;
    const int k = e % p, q = e / p;
    st_c(a.mpole, k + (size_t)p * (q + a.nrhs * (size_t)b), acc[t]);
  }
}

// M2M: each non-leaf box of a level pulls its four children's expansions.
__global__ void __launch_bounds__(kFmmThreads) m2m_kernel(FmmArgs a, const int* children) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int P = a.boxes[blockIdx.x];
  if (a.pcount[P] > 0 || children[4 * P] < 0) return;  // leaf: filled by P2M
  const int p = a.p;
  Cx* dp = reinterpret_cast<Cx*>(smem);  // 4 x p powers of (z_C - z_P) / s_P
  const double isp = rcp(a.side[P]);
  if (threadIdx.x < 4) {
    const int C = children[4 * P + threadIdx.x];
    const Cx d = {(a.cx[C] - a.cx[P]) * isp, (a.cy[C] - a.cy[P]) * isp};
    Cx v = {1.0, 0.0};
    for (int m = 0; m < p; ++m) {
      dp[threadIdx.x * p + m] = v;
      v = cmul(v, d);
    }
  }
  __syncthreads();
  const int P2 = 2 * p;
  for (int e = threadIdx.x; e < p * a.nrhs; e += blockDim.x) {
    const int l = e % p, q = e / p;
    Cx acc = {0.0, 0.0};
    for (int c = 0; c < 4; ++c) {
      const int C = children[4 * P + c];
      const double* M = a.mpole + 2 * (size_t)p * (q + a.nrhs * (size_t)C);
      double half = 1.0;
      for (int k = 0; k <= l; ++k) {
        const double f = a.binom[l * P2 + k] * half;
        acc = cadd(acc, cscale(cmul(ld_c(M, k), dp[c * p + l - k]), f));
        half *= 0.5;
      }
    }
    st_c(a.mpole, l + (size_t)p * (q + a.nrhs * (size_t)P), acc);
  }
}

// M2L from the V list and P2L from the X list; writes the box's local expansion.
__global__ void __launch_bounds__(kFmmThreads) m2l_kernel(FmmArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int B = a.boxes[blockIdx.x];
  const int p = a.p, nrhs = a.nrhs, P2 = 2 * p;
  Cx* av = reinterpret_cast<Cx*>(smem);      // p x nrhs scaled source coefficients
  Cx* vp = av + (size_t)p * nrhs;            // p: (-1)^l (s_B/d)^l / d
  Cx* pw = vp + p;                           // 64 x p powers for P2L
  const double zbx = a.cx[B], zby = a.cy[B], sB = a.side[B];
  constexpr int kPer = 4;  // (l, q) pairs per thread (p * nrhs <= 512)
  Cx acc[kPer];
#pragma unroll
  for (int t = 0; t < kPer; ++t) acc[t] = {0.0, 0.0};
  for (int vi = a.v_off[B]; vi < a.v_off[B + 1]; ++vi) {
    const int C = a.v_idx[vi];
    const Cx d = {zbx - a.cx[C], zby - a.cy[C]};
    const Cx id = cinv(d);
    if (threadIdx.x < 2) {
      // thread 0: u^k (u = s_C / d) into pw; thread 1: vp
      if (threadIdx.x == 0) {
        const Cx u = cscale(id, a.side[C]);
        Cx v = {1.0, 0.0};
        for (int k = 0; k < p; ++k) {
          pw[k] = v;
          v = cmul(v, u);
        }
      } else {
        const Cx w = cscale(id, sB);
        Cx v = id;
        for (int l = 0; l < p; ++l) {
          vp[l] = (l & 1) ? Cx{-v.re, -v.im} : v;
          v = cmul(v, w);
        }
      }
    }
    __syncthreads();
    const double* M = a.mpole + 2 * (size_t)p * nrhs * C;
    for (int e = threadIdx.x; e < p * nrhs; e += blockDim.x) {
      const int k = e % p, q = e / p;
      av[k + p * q] = cmul(ld_c(M, k + (size_t)p * q), pw[k]);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int e = threadIdx.x + t * blockDim.x;
      if (e >= p * nrhs) break;
      const int l = e % p, q = e / p;
      Cx s = {0.0, 0.0};
      const double* brow = a.binom + (size_t)l;  // C(k + l, l) = binom[(k + l) * P2 + l]
      for (int k = 0; k < p; ++k) {
        const double bk = brow[(size_t)(k + l) * P2];
        s.re += bk * av[k + p * q].re;
        s.im += bk * av[k + p * q].im;
      }
      acc[t] = cadd(acc[t], cmul(vp[l], s));
    }
    __syncthreads();
  }
  for (int xi = a.x_off[B]; xi < a.x_off[B + 1]; ++xi) {
    const int S = a.x_idx[xi];
    const int s0 = a.pstart[S], cnt = a.pcount[S];
    for (int j0 = 0; j0 < cnt; j0 += 64) {
      const int jc = cnt - j0 < 64 ? cnt - j0 : 64;
      for (int j = threadIdx.x; j < jc; j += blockDim.x) {
        const Cx w = {a.zx[s0 + j0 + j] - zbx, a.zy[s0 + j0 + j] - zby};
        const Cx iw = cinv(w);
        const Cx r = cscale(iw, sB);
        Cx v = iw;  // 1/w * r^l
        for (int l = 0; l < p; ++l) {
          pw[j * p + l] = v;
          v = cmul(v, r);
        }
      }
      __syncthreads();
#pragma unroll
      for (int t = 0; t < kPer; ++t) {
        const int e = threadIdx.x + t * blockDim.x;
        if (e >= p * nrhs) break;
        const int l = e % p, q = e / p;
        for (int j = 0; j < jc; ++j) {
          const Cx c = ld_c(a.charge, s0 + j0 + j + (size_t)a.npts * q);
          const Cx v = cmul(c, pw[j * p + l]);
          acc[t].re -= v.re;
          acc[t].im -= v.im;
        }
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int e = threadIdx.x + t * blockDim.x;
    if (e >= p * nrhs) break;
    const int l = e % p, q = e / p;
    st_c(a.local, l + (size_t)p * (q + nrhs * (size_t)B), acc[t]);
  }
}

// L2L: each box of a level adds its parent's shifted local expansion.
__global__ void __launch_bounds__(kFmmThreads) l2l_kernel(FmmArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int C = a.boxes[blockIdx.x];
  const int P = a.parent[C];
  if (P < 0) return;
  const int p = a.p, P2 = 2 * p;
  Cx* ep = reinterpret_cast<Cx*>(smem);
  if (threadIdx.x == 0) {
    const double isp = rcp(a.side[P]);
    const Cx e = {(a.cx[C] - a.cx[P]) * isp, (a.cy[C] - a.cy[P]) * isp};
    Cx v = {1.0, 0.0};
    for (int m = 0; m < p; ++m) {
      ep[m] = v;
      v = cmul(v, e);
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < p * a.nrhs; e += blockDim.x) {
    const int m = e % p, q = e / p;
    const double* Lp = a.local + 2 * (size_t)p * (q + a.nrhs * (size_t)P);
    Cx acc = {0.0, 0.0};
    for (int l = m; l < p; ++l) acc = cadd(acc, cscale(cmul(ld_c(Lp, l), ep[l - m]), a.binom[l * P2 + m]));
    acc = cscale(acc, ldexp(1.0, -m));
    const size_t o = m + (size_t)p * (q + a.nrhs * (size_t)C);
    st_c(a.local, o, cadd(ld_c(a.local, o), acc));
  }
}

// Evaluation at a leaf's points: L2P + M2P (W list) + P2P (U list).
__global__ void __launch_bounds__(kFmmThreads) eval_kernel(FmmArgs a, Geo<double> g,
                                                           const double* mu, double* y) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int B = a.boxes[blockIdx.x];
  const int s0 = a.pstart[B], cnt = a.pcount[B];
  const int p = a.p, nrhs = a.nrhs;
  double* sx = reinterpret_cast<double*>(smem);  // staged sources: 64 x (2 + 2 nrhs)
  double* sy = sx + 64;
  double* sc = sy + 64;                          // 64 x nrhs complex
  const double zbx = a.cx[B], zby = a.cy[B], isB = rcp(a.side[B]);
  for (int j0 = 0; j0 < cnt; j0 += blockDim.x) {
    const int j = j0 + threadIdx.x;
    const bool act = j < cnt;
    double phi[kMaxRhs];
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) phi[q] = 0.0;
    double tx = 0, ty = 0;
    if (act) {
      tx = a.zx[s0 + j];
      ty = a.zy[s0 + j];
      // L2P (Horner on the real part at the end)
      const Cx rho = {(tx - zbx) * isB, (ty - zby) * isB};
      for (int q = 0; q < nrhs; ++q) {
        const double* L = a.local + 2 * (size_t)p * (q + nrhs * (size_t)B);
        Cx h = ld_c(L, p - 1);
        for (int l = p - 2; l >= 0; --l) h = cadd(cmul(h, rho), ld_c(L, l));
        phi[q] += h.re;
      }
      // M2P from the W list
      for (int wi = a.w_off[B]; wi < a.w_off[B + 1]; ++wi) {
        const int C = a.w_idx[wi];
        const Cx w = {tx - a.cx[C], ty - a.cy[C]};
        const Cx iw = cinv(w);
        const Cx t = cscale(iw, a.side[C]);
        for (int q = 0; q < nrhs; ++q) {
          const double* M = a.mpole + 2 * (size_t)p * (q + nrhs * (size_t)C);
          Cx h = ld_c(M, p - 1);
          for (int k = p - 2; k >= 0; --k) h = cadd(cmul(h, t), ld_c(M, k));
          phi[q] += cmul(h, iw).re;
        }
      }
    }
    // P2P from the U list (sources staged 64 at a time)
    for (int ui = a.u_off[B]; ui < a.u_off[B + 1]; ++ui) {
      const int D = a.u_idx[ui];
      const int d0 = a.pstart[D], dcnt = a.pcount[D];
      for (int i0 = 0; i0 < dcnt; i0 += 64) {
        const int ic = dcnt - i0 < 64 ? dcnt - i0 : 64;
        __syncthreads();
        for (int e = threadIdx.x; e < ic; e += blockDim.x) {
          sx[e] = a.zx[d0 + i0 + e];
          sy[e] = a.zy[d0 + i0 + e];
        }
        for (int e = threadIdx.x; e < ic * nrhs; e += blockDim.x) {
          const int i = e % ic, q = e / ic;
          const size_t src = d0 + i0 + i + (size_t)a.npts * q;
          sc[2 * (i + 64 * q)] = a.charge[2 * src];
          sc[2 * (i + 64 * q) + 1] = a.charge[2 * src + 1];
        }
        __syncthreads();
        if (act) {
          for (int i = 0; i < ic; ++i) {
            if (d0 + i0 + i == s0 + j) continue;  // self
            const Cx iv = cinv(Cx{tx - sx[i], ty - sy[i]});
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q)
              if (q < nrhs) phi[q] += sc[2 * (i + 64 * q)] * iv.re - sc[2 * (i + 64 * q) + 1] * iv.im;
          }
        }
      }
    }
    if (act) {
      const int pt = a.slot_pt[s0 + j];
      const double diag = 0.5 + 0.5 * g.kap[pt] * g.w[pt] * (1.0 / (2.0 * CUDART_PI));
      for (int q = 0; q < nrhs; ++q)
        y[pt + (size_t)a.npts * q] = diag * mu[pt + (size_t)a.npts * q] + phi[q];
    }
  }
}

}  // namespace

cudaError_t fmm_laplace_apply(FmmPlan& f, const Geo<double>& geo, const double* mu, int nrhs,
                              double* y, cudaStream_t st) {
  if (!f.built) return cudaErrorInvalidValue;
  const int p = f.p, npts = f.npts, nb = f.nbox;
  if (p < 2 || p * kMaxRhs > 4 * kFmmThreads) return cudaErrorInvalidValue;
  set_smem_once<p2m_kernel>();
  set_smem_once<m2l_kernel>();
  for (int q0 = 0; q0 < nrhs; q0 += kMaxRhs) {
    const int nq = nrhs - q0 < kMaxRhs ? nrhs - q0 : kMaxRhs;
    cudaError_t e;
    if ((e = f.charge.ensure(2 * (size_t)npts * kMaxRhs)) != cudaSuccess) return e;
    if ((e = f.mpole.ensure(2 * (size_t)p * kMaxRhs * nb)) != cudaSuccess) return e;
    if ((e = f.local.ensure(2 * (size_t)p * kMaxRhs * nb)) != cudaSuccess) return e;
    FmmArgs a{};
    a.cx = f.cx.p;
    a.cy = f.cy.p;
    a.side = f.side.p;
    a.zx = f.zx.p;
    a.zy = f.zy.p;
    a.binom = f.binom.p;
    a.pstart = f.pstart.p;
    a.pcount = f.pcount.p;
    a.parent = f.parent.p;
    a.slot_pt = f.slot_pt.p;
    a.v_off = f.v_off.p;
    a.v_idx = f.v_idx.p;
    a.w_off = f.w_off.p;
    a.w_idx = f.w_idx.p;
    a.x_off = f.x_off.p;
    a.x_idx = f.x_idx.p;
    a.u_off = f.u_off.p;
    a.u_idx = f.u_idx.p;
    a.p = p;
    a.npts = npts;
    a.nrhs = nq;
    a.charge = f.charge.p;
    a.mpole = f.mpole.p;
    a.local = f.local.p;
    const double* muq = mu + (size_t)npts * q0;
    double* yq = y + (size_t)npts * q0;
    const size_t tot = (size_t)npts * nq;
    charges_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(geo, f.slot_pt.p, npts, muq, nq,
                                                                  f.charge.p);
    // upward pass
    a.boxes = f.leaves.p;
    p2m_kernel<<<(unsigned)f.leaves_h.size(), kFmmThreads, sizeof(Cx) * 64 * (size_t)p, st>>>(a);
    for (int lv = f.nlevels - 2; lv >= 0; --lv) {
      const int cnt = f.level_off[lv + 1] - f.level_off[lv];
      if (!cnt) continue;
      a.boxes = f.lvl_boxes.p + f.level_off[lv];
      m2m_kernel<<<cnt, kFmmThreads, sizeof(Cx) * 4 * p, st>>>(a, f.children.p);
    }
    // interactions and downward pass
    if ((e = cudaMemsetAsync(f.local.p, 0, 2 * sizeof(double) * (size_t)p * nq * nb, st)) != cudaSuccess)
      return e;
    if (!f.m2l_boxes_h.empty()) {
      a.boxes = f.m2l_boxes.p;
      m2l_kernel<<<(unsigned)f.m2l_boxes_h.size(), kFmmThreads,
                   sizeof(Cx) * ((size_t)p * nq + p + 64 * (size_t)p), st>>>(a);
    }
    for (int lv = 1; lv < f.nlevels; ++lv) {
      const int cnt = f.level_off[lv + 1] - f.level_off[lv];
      if (!cnt) continue;
      a.boxes = f.lvl_boxes.p + f.level_off[lv];
      l2l_kernel<<<cnt, kFmmThreads, sizeof(Cx) * p, st>>>(a);
    }
    a.boxes = f.leaves.p;
    eval_kernel<<<(unsigned)f.leaves_h.size(), kFmmThreads,
                  sizeof(double) * (128 + 2 * 64 * kMaxRhs), st>>>(a, geo, muq, yq);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace rskel
