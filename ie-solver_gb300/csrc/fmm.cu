// Fast multipole kernels for the Laplace double-layer product; see fmm.hpp
// for the formulation.  Templated on the number type R: double, float, or
// DF (float-float); complex numbers are (re, im) pairs of R.  Geometry comes
// in as FP64 box centres and leaf-relative point coordinates, so only box
// offsets (one per box pair) touch FP64.
//
// Scaled expansions for a box with centre z_B and side s_B:
//   multipole  phi(z) = sum_k  M_k s^k / (z - z_B)^(k+1)
//   local      phi(z) = sum_l  L_l ((z - z_B) / s)^l
// Translations (d = z_B - z_C for M2L, e = z_child - z_parent):
//   P2M  M_k = sum_j c_j ((z_j - z_B) / s_B)^k
//   M2M  M_l(P) = sum_{k<=l} M_k(C) C(l,k) (s_C/s_P)^k ((z_C - z_P)/s_P)^(l-k)
//        (s_C/s_P = 1/2 in a quadtree)
//   M2L  L_l(B) = (-1)^l (s_B/d)^l / d * sum_k C(k+l,l) M_k(C) (s_C/d)^k
//   L2L  L_m(C) = sum_{l>=m} L_l(P) C(l,m) (s_C/s_P)^m (e/s_P)^(l-m)
//   P2L  L_l(B) -= c_j / w (s_B / w)^l,       w = z_j - z_B
//   L2P  phi(z) = sum_l L_l ((z - z_B)/s_B)^l
//   M2P  phi(z) = (1/w) sum_k M_k (s_C / w)^k, w = z - z_C
#include <cuda_runtime.h>
#include <math_constants.h>

#include <type_traits>

#include "common.cuh"
#include "fmm.hpp"

namespace rskel {

namespace {

constexpr int kFmmThreads = 128;
constexpr int kMaxRhs = 8;  // right-hand sides per pass (larger batches loop)
constexpr int kStage = 64;  // points staged in shared memory at a time
constexpr int kEvalThreads = 128;

// Float-float numbers: value = hi + lo with |lo| <= ulp(hi)/2, ~48-bit
// significands.  Error-free transformations (Knuth's two-sum, and the
// product error from an explicit fused multiply-add; Dekker 1971), so the
// operations run on the FP32 pipes.
struct DF {
  float hi, lo;
  DF() = default;
  __host__ __device__ constexpr DF(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ explicit DF(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ explicit DF(int v) : DF((double)v) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ DF df_renorm(float s, float e) {
  const float h = s + e;
  return DF(h, e - (h - s));
}
__device__ __forceinline__ DF operator+(DF a, DF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
  return df_renorm(s, e);
}
__device__ __forceinline__ DF operator-(DF a) { return DF(-a.hi, -a.lo); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator*(DF a, DF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_renorm(p, e);
}
__device__ __forceinline__ DF& operator+=(DF& a, DF b) { return a = a + b; }
__device__ __forceinline__ DF& operator-=(DF& a, DF b) { return a = a - b; }
__device__ __forceinline__ DF& operator*=(DF& a, DF b) { return a = a * b; }
// 1/a: an FP32 reciprocal refined by one Newton step in float-float (the
// float and double overloads come from common.cuh).
using ::rskel::rcp;
__device__ __forceinline__ DF rcp(DF a) {
  const DF y(__frcp_rn(a.hi), 0.f);
  const DF e = DF(1.f, 0.f) - a * y;
  return y + y * e;
}

// acc += x y for the near field's sums.  For float-float the product's
// error (an explicit fused multiply-add) and the sum's error (two-sum) are
// collected in acc.lo without renormalising after every term; acc_norm
// renormalises (after each source box, so acc.lo stays a few ulps of
// acc.hi) and is a no-op for the other number types.
template <class R>
__device__ __forceinline__ void acc_fma(R& acc, R x, R y) { acc += x * y; }
__device__ __forceinline__ void acc_fma(DF& acc, DF x, DF y) {
  const float p = x.hi * y.hi;
  const float pe = fmaf(x.hi, y.hi, -p) + fmaf(x.hi, y.lo, x.lo * y.hi);
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  acc.lo += ((acc.hi - (s - bb)) + (p - bb)) + pe;
  acc.hi = s;
}
template <class R>
__device__ __forceinline__ void acc_norm(R&) {}
__device__ __forceinline__ void acc_norm(DF& a) { a = df_renorm(a.hi, a.lo); }

// Warp broadcast of lane src's value (float-float: both parts).
__device__ __forceinline__ float shfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double shfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ DF shfl(DF v, int src) { return DF(shfl(v.hi, src), shfl(v.lo, src)); }

template <class R>
__device__ __forceinline__ R to_r(double v) { return R(v); }
template <>
__device__ __forceinline__ float to_r<float>(double v) { return (float)v; }

template <class R>
struct Cx {
  R re, im;
};
template <class R>
__device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class R>
__device__ __forceinline__ Cx<R> cadd(Cx<R> a, Cx<R> b) {
  return {a.re + b.re, a.im + b.im};
}
template <class R>
__device__ __forceinline__ Cx<R> csub(Cx<R> a, Cx<R> b) {
  return {a.re - b.re, a.im - b.im};
}
template <class R>
__device__ __forceinline__ Cx<R> cinv(Cx<R> a) {
  const R d = rcp(a.re * a.re + a.im * a.im);
  return {a.re * d, -a.im * d};
}
template <class R>
__device__ __forceinline__ Cx<R> cscale(Cx<R> a, R s) {
  return {a.re * s, a.im * s};
}

// Leaf-relative point positions: FP64, or a hi + lo float pair.
template <class R>
struct Pos {
  float hx, lx, hy, ly;
};
template <>
struct Pos<double> {
  double x, y;
};
__device__ __forceinline__ Cx<double> vec(Pos<double> a) { return {a.x, a.y}; }
__device__ __forceinline__ Cx<float> vec(Pos<float> a) { return {a.hx + a.lx, a.hy + a.ly}; }
__device__ __forceinline__ Cx<DF> vec(Pos<DF> a) { return {DF(a.hx, a.lx), DF(a.hy, a.ly)}; }
// t - s - off for points t, s of leaves whose centres differ by off = c_s - c_t.
// The near-field difference is a small remainder of O(side) terms, so the
// FP32 variant forms it in float-float too and rounds once at the end.
template <class R>
struct OffT {
  using type = DF;
};
template <>
struct OffT<double> {
  using type = double;
};
__device__ __forceinline__ Cx<double> diff(Pos<double> t, Pos<double> s, Cx<double> off) {
  return {(t.x - s.x) - off.re, (t.y - s.y) - off.im};
}
__device__ __forceinline__ Cx<DF> diff(Pos<DF> t, Pos<DF> s, Cx<DF> off) {
  return {(DF(t.hx, t.lx) - DF(s.hx, s.lx)) - off.re, (DF(t.hy, t.ly) - DF(s.hy, s.ly)) - off.im};
}
__device__ __forceinline__ Cx<float> diff(Pos<float> t, Pos<float> s, Cx<DF> off) {
  const DF x = (DF(t.hx, t.lx) - DF(s.hx, s.lx)) - off.re;
  const DF y = (DF(t.hy, t.ly) - DF(s.hy, s.ly)) - off.im;
  return {x.hi + x.lo, y.hi + y.lo};
}

template <class R>
struct FmmArgs {
  const double *cx, *cy, *side;
  const double *rx, *ry;                  // FP64 variant
  const float *rxh, *rxl, *ryh, *ryl;     // float and float-float variants
  const R* binom;
  int bs;  // row stride of binom: twice the order it was built for (at least a.p)
  const int *pstart, *pcount, *parent, *slot_pt, *children;
  const int *v_off, *v_idx, *w_off, *w_idx, *x_off, *x_idx, *u_off, *u_idx;
  const int* boxes;
  int p, npts, nrhs;  // nrhs: channels of this pass
  int mode;           // FmmMode
  const R* charge;  // complex, 2 * (slot + npts * q)
  R* mpole;         // complex, 2 * (k + p * (q + nrhs * box))
  R* local;
  // near-field source data in slot order, kSrcStride values of R per slot:
  // Laplace (mode 0) the charge factor b_j = -(w_j / 2pi) nu_j (complex)
  // then the nrhs densities; Neumann (mode 1) the nrhs real charges
  const R* src;
};
constexpr int kSrcStride = 2 + kMaxRhs;

__device__ __forceinline__ Pos<double> pt_pos(const FmmArgs<double>& a, int s) {
  return {a.rx[s], a.ry[s]};
}
template <class R>
__device__ __forceinline__ Pos<R> pt_pos(const FmmArgs<R>& a, int s) {
  return {a.rxh[s], a.rxl[s], a.ryh[s], a.ryl[s]};
}
// c_to - c_from in FP64, then in R
template <class R>
__device__ __forceinline__ Cx<R> box_off(const FmmArgs<R>& a, int from, int to) {
  return {to_r<R>(a.cx[to] - a.cx[from]), to_r<R>(a.cy[to] - a.cy[from])};
}
// the same offset in the near-field difference's number type
template <class R>
__device__ __forceinline__ Cx<typename OffT<R>::type> p2p_off(const FmmArgs<R>& a, int from, int to) {
  using T = typename OffT<R>::type;
  return {T(a.cx[to] - a.cx[from]), T(a.cy[to] - a.cy[from])};
}
template <class R>
__device__ __forceinline__ R side_of(const FmmArgs<R>& a, int b) {
  return to_r<R>(a.side[b]);
}

template <class R>
__device__ __forceinline__ Cx<R> ld_c(const R* a, size_t i) {
  return {a[2 * i], a[2 * i + 1]};
}
template <class R>
__device__ __forceinline__ void st_c(R* a, size_t i, Cx<R> v) {
  a[2 * i] = v.re;
  a[2 * i + 1] = v.im;
}

// Complex charges c_j = -(w_j / 2pi) (n_x + i n_y) mu_j in slot order; and
// the near-field source data (charge factor, densities in R) once per slot.
template <class R>
__global__ void charges_kernel(Geo<double> g, const int* slot_pt, int npts, const double* mu,
                               int nrhs, R* charge, R* src) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)npts * nrhs) return;
  const int s = (int)(e % npts), q = (int)(e / npts);
  const int pt = slot_pt[s];
  const double f = -g.w[pt] * (1.0 / (2.0 * CUDART_PI));
  const double m = mu[pt + (size_t)npts * q];
  charge[2 * e] = (R)(f * m * g.nx[pt]);
  charge[2 * e + 1] = (R)(f * m * g.ny[pt]);
  R* sr = src + (size_t)kSrcStride * s;
  if (q == 0) {
    sr[0] = to_r<R>(f * g.nx[pt]);
    sr[1] = to_r<R>(f * g.ny[pt]);
  }
  sr[2 + q] = to_r<R>(m);
}

// Neumann (adjoint double layer, kernel.cpp:80-91): real charges
// c_j = (w_j / 2pi) mu_j; (K mu)_i gets Re(nu_i sum_j c_j / (z_i - z_j)).
template <class R>
__global__ void neumann_charges_kernel(Geo<double> g, const int* slot_pt, int npts,
                                       const double* mu, int nrhs, R* charge, R* src) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)npts * nrhs) return;
  const int s = (int)(e % npts), q = (int)(e / npts);
  const int pt = slot_pt[s];
  const R c = to_r<R>(g.w[pt] * (1.0 / (2.0 * CUDART_PI)) * mu[pt + (size_t)npts * q]);
  charge[2 * e] = c;
  charge[2 * e + 1] = to_r<R>(0.0);
  src[(size_t)kSrcStride * s + 2 + q] = c;
}

// Stokes double layer in complex form.  With tau = z_i - z_j, nu_j the
// normal and mu_j = mu_x + i mu_y the density, the off-diagonal part of
// kernel.cpp:212-290, (w_j/pi) (r.n_j)(r.mu_j) r / |r|^4, is
//   a_j / tau + b_j / conj(tau) + conj(a_j) tau / conj(tau)^2,
//   a_j = (w_j / 4pi) nu_j mu_j,  b_j = (w_j / 2pi) Re(conj(nu_j) mu_j) (real).
// Summed over j that is S_A + conj(S_B) - conj((conj(z) - conj(c)) S_A' + G')
// for Cauchy sums S_A, S_B (charges a, b) and, about any centre c, the sum
// G(z) = sum_j a_j (conj(c) - conj(z_j)) / (z - z_j).  Three channels per
// density: A, B, and E with charges a_j conj(z_j - c_leaf) relative to the
// source leaf's centre; translations turn E into G with conjugated box
// offsets (M2M, M2L, L2L below), so no absolute coordinate enters.
template <class R>
__global__ void stokes_charges_kernel(Geo<double> g, const int* slot_pt, const double* rx,
                                      const double* ry, int npts, const double* mu, int nq,
                                      R* charge) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)npts * nq) return;
  const int s = (int)(e % npts), q = (int)(e / npts);
  const int pt = slot_pt[s];
  const size_t D = 2 * (size_t)npts;
  const double mx = mu[2 * (size_t)pt + D * q], my = mu[2 * (size_t)pt + 1 + D * q];
  const double nx = g.nx[pt], ny = g.ny[pt], f = g.w[pt] * (1.0 / (4.0 * CUDART_PI));
  const double ar = f * (nx * mx - ny * my), ai = f * (nx * my + ny * mx);
  const double b = 2.0 * f * (nx * mx + ny * my);
  const double er = ar * rx[s] + ai * ry[s], ei = ai * rx[s] - ar * ry[s];  // a conj(rel)
  const double v[6] = {ar, ai, b, 0.0, er, ei};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t o = s + (size_t)npts * (3 * q + c);
    charge[2 * o] = to_r<R>(v[2 * c]);
    charge[2 * o + 1] = to_r<R>(v[2 * c + 1]);
  }
}

// Per right-hand side, the rank-one part of the Neumann and Stokes operators:
// sum_j w_j mu_j (Neumann, kernel.cpp:80-91) or sum_j w_j n_j . mu_j (Stokes,
// the w n_t n_s term of kernel.cpp:212-290).  One block per right-hand side.
__global__ void rank1_kernel(Geo<double> g, int npts, const double* mu, int mode, double* out) {
  __shared__ double red[1024];
  const int q = blockIdx.x;
  double acc = 0.0;
  if (mode == 1) {
    for (int i = threadIdx.x; i < npts; i += blockDim.x) acc += g.w[i] * mu[i + (size_t)npts * q];
  } else {
    const size_t D = 2 * (size_t)npts;
    for (int i = threadIdx.x; i < npts; i += blockDim.x)
      acc += g.w[i] * (g.nx[i] * mu[2 * (size_t)i + D * q] + g.ny[i] * mu[2 * (size_t)i + 1 + D * q]);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[q] = red[0];
}

template <class R>
__device__ __forceinline__ Cx<R> cconj(Cx<R> a) {
  return {a.re, -a.im};
}
template <class R>
__device__ __forceinline__ bool is_g(const FmmArgs<R>& a, int q) {
  return a.mode == 2 && q % 3 == 2;
}

// P2M for every non-empty leaf (points staged kStage at a time).
template <class R>
__global__ void __launch_bounds__(kFmmThreads) p2m_kernel(FmmArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  pdl_launch_dependents();  // (the charges are read after pdl_wait below)
  const int b = a.boxes[blockIdx.x];
  const int s0 = a.pstart[b], cnt = a.pcount[b], p = a.p;
  Cx<R>* pw = reinterpret_cast<Cx<R>*>(smem);  // kStage x p
  const R is = rcp(side_of(a, b));
  constexpr int kPer = 4;  // (k, q) pairs per thread (p * nrhs <= 512)
  Cx<R> acc[kPer];
#pragma unroll
  for (int t = 0; t < kPer; ++t) acc[t] = {(R)0, (R)0};
  for (int j0 = 0; j0 < cnt; j0 += kStage) {
    const int jc = cnt - j0 < kStage ? cnt - j0 : kStage;
    __syncthreads();
    for (int j = threadIdx.x; j < jc; j += blockDim.x) {
      const Cx<R> rho = cscale(vec(pt_pos(a, s0 + j0 + j)), is);
      Cx<R> v = {(R)1, (R)0};
      for (int k = 0; k < p; ++k) {
        pw[j * p + k] = v;
        v = cmul(v, rho);
      }
    }
    __syncthreads();
    pdl_wait();
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

// M2M: each non-empty, non-leaf box of a level pulls its children's
// expansions.  With d = (z_C - z_P)/s_P and g = 1/(2d) the shift is
//   M_l(P) = sum_C d^l sum_{k<=l} C(l,k) (M_k(C) g^k),
// a real Pascal-matrix product between two diagonal complex scalings.
// Stokes E channels re-centre their charges a_j conj(z_j - c) on the
// parent: E(P) = shift(E(C)) + conj(z_C - z_P) shift(A(C)).
template <class R>
__global__ void __launch_bounds__(kFmmThreads) m2m_kernel(FmmArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  // (programmatic dependent launch: the offsets' powers below overlap the
  // previous level's kernel; its multipoles are read after pdl_wait)
  pdl_launch_dependents();
  const int P = a.boxes[blockIdx.x];
  if (a.pcount[P] > 0) return;  // leaf: filled by P2M
  const int p = a.p, nrhs = a.nrhs, P2 = a.bs;
  Cx<R>* dl = reinterpret_cast<Cx<R>*>(smem);  // 4 x p: d_c^l
  Cx<R>* gk = dl + 4 * p;                      // 4 x p: g_c^k
  Cx<R>* av = gk + 4 * p;                      // 4 x nrhs x p: M_k(c) g_c^k
  Cx<R>* oc = av + 4 * p * nrhs;               // 4: conj(z_C - z_P)
  const R isp = rcp(side_of(a, P));
  if (threadIdx.x < 4) {
    const int C = a.children[4 * P + threadIdx.x];
    if (C >= 0) oc[threadIdx.x] = cconj(box_off(a, P, C));
  }
  if (threadIdx.x < 8) {
    const int c = threadIdx.x & 3;
    const int C = a.children[4 * P + c];
    if (C >= 0) {
      const Cx<R> d = cscale(box_off(a, P, C), isp);
      const Cx<R> base = threadIdx.x < 4 ? d : cinv(cscale(d, (R)2));
      Cx<R>* out = (threadIdx.x < 4 ? dl : gk) + c * p;
      Cx<R> v = {(R)1, (R)0};
      for (int m = 0; m < p; ++m) {
        out[m] = v;
        v = cmul(v, base);
      }
    }
  }
  __syncthreads();
  pdl_wait();
  for (int e = threadIdx.x; e < 4 * p * nrhs; e += blockDim.x) {
    const int k = e % p, q = (e / p) % nrhs, c = e / (p * nrhs);
    const int C = a.children[4 * P + c];
    av[e] = C >= 0 ? cmul(ld_c(a.mpole, k + (size_t)p * (q + nrhs * (size_t)C)), gk[c * p + k])
                   : Cx<R>{(R)0, (R)0};
  }
  __syncthreads();
  for (int e = threadIdx.x; e < p * nrhs; e += blockDim.x) {
    const int l = e % p, q = e / p;
    Cx<R> acc = {(R)0, (R)0};
    for (int c = 0; c < 4; ++c) {
      if (a.children[4 * P + c] < 0) continue;
      const Cx<R>* ac = av + (size_t)p * (q + nrhs * c);
      Cx<R> t = {(R)0, (R)0};
      for (int k = 0; k <= l; ++k) {
        const R bk = a.binom[l * P2 + k];
        t.re += bk * ac[k].re;
        t.im += bk * ac[k].im;
      }
      if (is_g(a, q)) {
        const Cx<R>* aa = av + (size_t)p * (q - 2 + nrhs * c);
        Cx<R> ta = {(R)0, (R)0};
        for (int k = 0; k <= l; ++k) {
          const R bk = a.binom[l * P2 + k];
          ta.re += bk * aa[k].re;
          ta.im += bk * aa[k].im;
        }
        t = cadd(t, cmul(oc[c], ta));
      }
      acc = cadd(acc, cmul(dl[c * p + l], t));
    }
    st_c(a.mpole, l + (size_t)p * (q + nrhs * (size_t)P), acc);
  }
}

// M2L from the V list and P2L from the X list; writes the box's local expansion.
// Stokes G channels: G(B) gets conj(c_B - c_C) M2L(A(C)) - M2L(E(C)) from a
// V-list box, and charges -a_j conj(z_j - c_B) from an X-list box's points.
template <class R>
__global__ void __launch_bounds__(kFmmThreads) m2l_kernel(FmmArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int B = a.boxes[blockIdx.x];
  const int p = a.p, nrhs = a.nrhs, P2 = a.bs;
  Cx<R>* av = reinterpret_cast<Cx<R>*>(smem);  // p x nrhs scaled source coefficients
  Cx<R>* vp = av + (size_t)p * nrhs;           // p: (-1)^l (s_B/d)^l / d
  Cx<R>* pw = vp + p;                          // kStage x p powers for P2L
  Cx<R>* ws = pw + kStage * (size_t)p;         // kStage: conj(z_j - c_B) (Stokes X list)
  Cx<R>* dcs = ws + kStage;                    // 1: conj(c_B - c_C) (Stokes V list)
  const R sB = side_of(a, B);
  constexpr int kPer = 4;  // (l, q) pairs per thread (p * nrhs <= 512)
  Cx<R> acc[kPer];
#pragma unroll
  for (int t = 0; t < kPer; ++t) acc[t] = {(R)0, (R)0};
  for (int vi = a.v_off[B]; vi < a.v_off[B + 1]; ++vi) {
    const int C = a.v_idx[vi];
    if (threadIdx.x < 2) {
      const Cx<R> id = cinv(box_off(a, C, B));
      // thread 0: u^k (u = s_C / d) into pw; thread 1: vp
      if (threadIdx.x == 0) {
        dcs[0] = cconj(box_off(a, C, B));
        const Cx<R> u = cscale(id, side_of(a, C));
        Cx<R> v = {(R)1, (R)0};
        for (int k = 0; k < p; ++k) {
          pw[k] = v;
          v = cmul(v, u);
        }
      } else {
        const Cx<R> w = cscale(id, sB);
        Cx<R> v = id;
        for (int l = 0; l < p; ++l) {
          vp[l] = (l & 1) ? Cx<R>{-v.re, -v.im} : v;
          v = cmul(v, w);
        }
      }
    }
    __syncthreads();
    const R* M = a.mpole + 2 * (size_t)p * nrhs * C;
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
      Cx<R> s = {(R)0, (R)0};
      const R* brow = a.binom + (size_t)l;  // C(k + l, l) = binom[(k + l) * bs + l]
      for (int k = 0; k < p; ++k) {
        const R bk = brow[(size_t)(k + l) * P2];
        s.re += bk * av[k + p * q].re;
        s.im += bk * av[k + p * q].im;
      }
      if (is_g(a, q)) {
        Cx<R> sa = {(R)0, (R)0};
        for (int k = 0; k < p; ++k) {
          const R bk = brow[(size_t)(k + l) * P2];
          sa.re += bk * av[k + p * (q - 2)].re;
          sa.im += bk * av[k + p * (q - 2)].im;
        }
        s = csub(cmul(dcs[0], sa), s);
      }
      acc[t] = cadd(acc[t], cmul(vp[l], s));
    }
    __syncthreads();
  }
  for (int xi = a.x_off[B]; xi < a.x_off[B + 1]; ++xi) {
    const int S = a.x_idx[xi];
    const int s0 = a.pstart[S], cnt = a.pcount[S];
    const Cx<R> offS = box_off(a, B, S);  // z_j - z_B = (z_j - c_S) + (c_S - c_B)
    for (int j0 = 0; j0 < cnt; j0 += kStage) {
      const int jc = cnt - j0 < kStage ? cnt - j0 : kStage;
      for (int j = threadIdx.x; j < jc; j += blockDim.x) {
        const Cx<R> w = cadd(vec(pt_pos(a, s0 + j0 + j)), offS);
        const Cx<R> iw = cinv(w);
        ws[j] = cconj(w);
        const Cx<R> r = cscale(iw, sB);
        Cx<R> v = iw;  // 1/w * r^l
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
        if (is_g(a, q)) {  // charges -a_j conj(w_j)
          for (int j = 0; j < jc; ++j) {
            const Cx<R> c = cmul(ld_c(a.charge, s0 + j0 + j + (size_t)a.npts * (q - 2)), ws[j]);
            acc[t] = cadd(acc[t], cmul(c, pw[j * p + l]));
          }
        } else {
          for (int j = 0; j < jc; ++j) {
            const Cx<R> v = cmul(ld_c(a.charge, s0 + j0 + j + (size_t)a.npts * q), pw[j * p + l]);
            acc[t].re -= v.re;
            acc[t].im -= v.im;
          }
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

// L2L: each non-empty box of a level adds its parent's shifted local
// expansion.  With e = (z_C - z_P)/s_P the shift is
//   L_m(C) += (2e)^-m sum_{l>=m} C(l,m) (L_l(P) e^l).
// Stokes G channels re-centre on the child: G(C) += shift(G(P)) +
// conj(z_C - z_P) shift(A(P)).
template <class R>
__global__ void __launch_bounds__(kFmmThreads) l2l_kernel(FmmArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  pdl_launch_dependents();  // (as in m2m_kernel)
  const int C = a.boxes[blockIdx.x];
  const int P = a.parent[C];
  if (P < 0) return;
  const int p = a.p, nrhs = a.nrhs, P2 = a.bs;
  Cx<R>* el = reinterpret_cast<Cx<R>*>(smem);  // p: e^l
  Cx<R>* hm = el + p;                          // p: (2e)^-m
  Cx<R>* bv = hm + p;                          // nrhs x p: L_l(P) e^l
  const Cx<R> ocp = cconj(box_off(a, P, C));
  if (threadIdx.x < 2) {
    const Cx<R> e = cscale(box_off(a, P, C), rcp(side_of(a, P)));
    const Cx<R> base = threadIdx.x == 0 ? e : cinv(cscale(e, (R)2));
    Cx<R>* out = threadIdx.x == 0 ? el : hm;
    Cx<R> v = {(R)1, (R)0};
    for (int m = 0; m < p; ++m) {
      out[m] = v;
      v = cmul(v, base);
    }
  }
  __syncthreads();
  pdl_wait();
  for (int e = threadIdx.x; e < p * nrhs; e += blockDim.x) {
    const int l = e % p, q = e / p;
    bv[e] = cmul(ld_c(a.local, l + (size_t)p * (q + nrhs * (size_t)P)), el[l]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < p * nrhs; e += blockDim.x) {
    const int m = e % p, q = e / p;
    const Cx<R>* bq = bv + (size_t)p * q;
    Cx<R> t = {(R)0, (R)0};
    for (int l = m; l < p; ++l) {
      const R bl = a.binom[l * P2 + m];
      t.re += bl * bq[l].re;
      t.im += bl * bq[l].im;
    }
    if (is_g(a, q)) {
      const Cx<R>* ba = bv + (size_t)p * (q - 2);
      Cx<R> ta = {(R)0, (R)0};
      for (int l = m; l < p; ++l) {
        const R bl = a.binom[l * P2 + m];
        ta.re += bl * ba[l].re;
        ta.im += bl * ba[l].im;
      }
      t = cadd(t, cmul(ocp, ta));
    }
    const size_t o = m + (size_t)p * (q + nrhs * (size_t)C);
    st_c(a.local, o, cadd(ld_c(a.local, o), cmul(hm[m], t)));
  }
}

// Evaluation at a leaf's points: L2P + M2P (W list) + P2P (U list), then
// y = ya * y + yb * (diag mu + phi) (Laplace double layer; for Neumann, phi
// is Re of the target normal times the Cauchy sum, plus the rank-one sum).
// One CTA of kEvalWarps warps per leaf, one lane per target: the target's
// sums for every right-hand side stay in registers; the warps split the
// work on the same 32 targets (L2P and M2P by right-hand side, P2P by
// source, round robin) and add their partial sums in a fixed order at the
// end.  Each source's data (position, charge factor, densities, written once
// per product by the charges kernel) is read by a whole warp at one
// address, so no shared-memory staging and no barrier sit in the pair loop.
// A leaf of more than 32 points takes several passes.
// kPart 0 does all of it.  With the product split over two streams:
// kPart 1 does only the near field (P2P) and stores its sums per (slot,
// right-hand side) in nearsum, as soon as the sources are written; kPart 3
// does only M2P over the W list and adds its sums to nearsum, as soon as
// the upward pass is done; kPart 2 does L2P after the downward pass, adds
// nearsum and finishes.  Only the last is on the product's critical path.
// The FP32 products, whose passes are short, keep M2P with L2P (kPart 4):
// there the side stream's M2P finished after the downward pass.
constexpr int kEvalWarps = 4;
enum EvalPart : int { kEvalAll = 0, kEvalNear = 1, kEvalFar = 2, kEvalW = 3, kEvalFarW = 4 };
template <class R, int kPart>
__global__ void __launch_bounds__(32 * kEvalWarps) eval_warp_kernel(
    FmmArgs<R> a, Geo<double> g, const double* mu, double* y, double ya, double yb,
    const double* r1, double* nearsum, int nbox) {
  __shared__ double part[kEvalWarps - 1][32][kMaxRhs];
  // each warp's copy of the expansions it evaluates (two right-hand sides of
  // one box, orders up to 64): the Horner chains below then read shared
  // memory, not a global load per step
  __shared__ R wexp[kPart == kEvalNear ? 1 : kEvalWarps][4 * 64];
  pdl_launch_dependents();  // (expansions are read after pdl_wait below)
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  // one leaf per CTA, or (a grid smaller than the leaf count) leaves
  // blockIdx.x, + gridDim.x, ...
  for (int li = blockIdx.x; li < nbox; li += gridDim.x) {
  const int B = a.boxes[li];
  const int s0 = a.pstart[B], cnt = a.pcount[B];
  const int p = a.p, nrhs = a.nrhs;
  const R isB = rcp(side_of(a, B));
  for (int j0 = 0; j0 < cnt; j0 += 32) {
    const int j = j0 + lane;
    const bool act = j < cnt;
    const int ts = s0 + (act ? j : 0);  // an idle lane shadows the leaf's first point
    R phi[kMaxRhs];
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) phi[q] = (R)0;
    const Pos<R> tp = pt_pos(a, ts);
    Cx<R> tnu = {(R)1, (R)0};
    if (a.mode == 1) {
      const int pt = a.slot_pt[ts];
      tnu = {to_r<R>(g.nx[pt]), to_r<R>(g.ny[pt])};
    }
    pdl_wait();
    R* wx = wexp[kPart == kEvalNear ? 0 : wp];
    R* wy = wx + 2 * p;
    if constexpr (kPart == kEvalAll || kPart == kEvalFar || kPart == kEvalFarW) {
    // L2P (right-hand sides q = wp, wp + kEvalWarps, ...; two of them at a
    // time, whose Horner chains interleave; the loop is kept rolled and its
    // results added through an unrolled select, which keeps the kernel's
    // code small)
    const Cx<R> rho = cscale(vec(tp), isB);
#pragma unroll 1
    for (int qq = wp; qq < nrhs; qq += 2 * kEvalWarps) {
      const int q2 = qq + kEvalWarps;
      const bool two = q2 < nrhs;
      const R* L = a.local + 2 * (size_t)p * (qq + nrhs * (size_t)B);
      __syncwarp();  // the previous expansions' reads are done
      for (int e = lane; e < 2 * p; e += 32) wx[e] = L[e];
      if (two)
        for (int e = lane; e < 2 * p; e += 32) wy[e] = L[2 * (size_t)p * kEvalWarps + e];
      __syncwarp();
      Cx<R> h = ld_c(wx, p - 1), g2 = two ? ld_c(wy, p - 1) : Cx<R>{(R)0, (R)0};
      for (int l = p - 2; l >= 0; --l) {
        h = cadd(cmul(h, rho), ld_c(wx, l));
        if (two) g2 = cadd(cmul(g2, rho), ld_c(wy, l));
      }
      const R v = cmul(tnu, h).re, v2 = cmul(tnu, g2).re;
#pragma unroll
      for (int q = 0; q < kMaxRhs; ++q) {
        if (q == qq) phi[q] += v;
        if (two && q == q2) phi[q] += v2;
      }
    }
    }  // L2P
    if constexpr (kPart == kEvalAll || kPart == kEvalW || kPart == kEvalFarW) {
    // M2P from the W list (the same split by right-hand side; with fewer
    // right-hand sides than warps, the warps of one right-hand side take
    // every G-th box of the list).  Box offsets and sides need FP64
    // arithmetic (slow on this GPU), so lane l forms them for the list's l-th
    // box and the warp broadcasts them in turn.
    const int nr = nrhs < kEvalWarps ? nrhs : kEvalWarps;
    const int G = kEvalWarps / nr, grp = wp / nr, rq = wp % nr;
    if (grp < G)
    for (int wb = a.w_off[B]; wb < a.w_off[B + 1]; wb += 32) {
      const int nwb = min(32, a.w_off[B + 1] - wb);
      int Cl = 0;
      Cx<R> ol = {(R)0, (R)0};
      R sl = (R)1;
      if (lane < nwb) {
        Cl = a.w_idx[wb + lane];
        ol = box_off(a, Cl, B);
        sl = side_of(a, Cl);
      }
      for (int t = 0; t < nwb; ++t) {
        if ((wb + t) % G != grp) continue;  // (warp-uniform)
        const int C = __shfl_sync(0xffffffffu, Cl, t);
        const Cx<R> oc = {shfl(ol.re, t), shfl(ol.im, t)};
        const R sc = shfl(sl, t);
        const Cx<R> iw = cinv(cadd(vec(tp), oc));  // z - c_C
        const Cx<R> tw = cscale(iw, sc);
#pragma unroll 1
        for (int qq = rq; qq < nrhs; qq += 2 * kEvalWarps) {
          const int q2 = qq + kEvalWarps;
          const bool two = q2 < nrhs;
          const R* M = a.mpole + 2 * (size_t)p * (qq + nrhs * (size_t)C);
          __syncwarp();
          for (int e = lane; e < 2 * p; e += 32) wx[e] = M[e];
          if (two)
            for (int e = lane; e < 2 * p; e += 32) wy[e] = M[2 * (size_t)p * kEvalWarps + e];
          __syncwarp();
          Cx<R> h = ld_c(wx, p - 1), g2 = two ? ld_c(wy, p - 1) : Cx<R>{(R)0, (R)0};
          for (int k = p - 2; k >= 0; --k) {
            h = cadd(cmul(h, tw), ld_c(wx, k));
            if (two) g2 = cadd(cmul(g2, tw), ld_c(wy, k));
          }
          const R v = cmul(tnu, cmul(h, iw)).re, v2 = cmul(tnu, cmul(g2, iw)).re;
#pragma unroll
          for (int q = 0; q < kMaxRhs; ++q) {
            if (q == qq) phi[q] += v;
            if (two && q == q2) phi[q] += v2;
          }
        }
      }
    }
    }  // M2P
    if constexpr (kPart == kEvalAll || kPart == kEvalNear) {
    // P2P from the U list: this warp takes every kEvalWarps-th source
    // (offsets broadcast as above)
    using OT = typename OffT<R>::type;
    int rr = wp;  // the source's position in the U list's concatenation, mod kEvalWarps
    for (int ub = a.u_off[B]; ub < a.u_off[B + 1]; ub += 32) {
      const int nub = min(32, a.u_off[B + 1] - ub);
      int Dl = 0;
      Cx<OT> ol = {OT(0.0), OT(0.0)};
      if (lane < nub) {
        Dl = a.u_idx[ub + lane];
        ol = p2p_off(a, B, Dl);
      }
      for (int t = 0; t < nub; ++t) {
        const int D = __shfl_sync(0xffffffffu, Dl, t);
        const Cx<OT> offD = {shfl(ol.re, t), shfl(ol.im, t)};
        const int d0 = a.pstart[D], dc = a.pcount[D];
        int sj = d0 + rr;
        for (; sj < d0 + dc; sj += kEvalWarps) {
          if (sj == ts) continue;  // self
          Cx<R> iv = cinv(diff(tp, pt_pos(a, sj), offD));
          const R* sr = a.src + (size_t)kSrcStride * sj;
          if (a.mode == 0) {
            const R tr = sr[0] * iv.re - sr[1] * iv.im;
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q)
              if (q < nrhs) acc_fma(phi[q], sr[2 + q], tr);
          } else {
            iv = cmul(tnu, iv);
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q)
              if (q < nrhs) acc_fma(phi[q], sr[2 + q], iv.re);
          }
        }
        rr = sj - (d0 + dc);  // carried into the next source box
#pragma unroll
        for (int q = 0; q < kMaxRhs; ++q) acc_norm(phi[q]);
      }
    }
    }  // near field
    // partial sums of warps 1.. to warp 0, added in warp order
    __syncthreads();
    if (wp > 0)
#pragma unroll
      for (int q = 0; q < kMaxRhs; ++q) part[wp - 1][lane][q] = (double)phi[q];
    __syncthreads();
    if (wp == 0 && act && (kPart == kEvalNear || kPart == kEvalW)) {
#pragma unroll
      for (int q = 0; q < kMaxRhs; ++q) {
        if (q < nrhs) {
          double tot = (double)phi[q];
          for (int w = 1; w < kEvalWarps; ++w) tot += part[w - 1][lane][q];
          double* o = nearsum + ts + (size_t)a.npts * q;
          *o = kPart == kEvalW ? *o + tot : tot;
        }
      }
    } else if (wp == 0 && act) {
      const int pt = a.slot_pt[ts];
      const double diag = (a.mode == 1 ? -0.5 : 0.5) +
                          0.5 * g.kap[pt] * g.w[pt] * (1.0 / (2.0 * CUDART_PI));
#pragma unroll
      for (int q = 0; q < kMaxRhs; ++q) {
        if (q < nrhs) {
          double tot = (double)phi[q];
          for (int w = 1; w < kEvalWarps; ++w) tot += part[w - 1][lane][q];
          if (kPart == kEvalFar || kPart == kEvalFarW) tot += nearsum[ts + (size_t)a.npts * q];
          const size_t o = pt + (size_t)a.npts * q;
          const double v = yb * (diag * mu[o] + tot + (a.mode == 1 ? r1[q] : 0.0));
          y[o] = ya == 0.0 ? v : ya * y[o] + v;
        }
      }
    }
  }
  }  // leaves
}

// Stokes evaluation at a leaf's points (channels A, B, G of up to
// kMaxDens densities): with rho = (z - c_B)/s_B,
//   u = S_A + conj(S_B) - conj(conj(rho) dS_A/drho + dG/dz)   (local part)
// plus, per W-list box C (w = z - c_C), S_A + conj(S_B) +
// conj(S_E' - conj(w) S_A'), and per U-list source the direct
// a/tau + b/conj(tau) + conj(a conj(tau) / tau^2); then the diagonal
// -mu/2 + pot t (t . mu) (pot = -kappa w / 2pi, t the tangent) and the
// rank-one n_i sum_j w_j n_j . mu_j of kernel.cpp:212-290.
constexpr int kMaxDens = kMaxRhs / 3;
template <class R>
__global__ void __launch_bounds__(kEvalThreads, 4) stokes_eval_kernel(FmmArgs<R> a,
                                                                      Geo<double> g,
                                                                      const double* mu,
                                                                      double* y, double ya,
                                                                      double yb,
                                                                      const double* r1) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int B = a.boxes[blockIdx.x];
  const int s0 = a.pstart[B], cnt = a.pcount[B];
  const int p = a.p, nch = a.nrhs, nq = nch / 3;
  Pos<R>* sp = reinterpret_cast<Pos<R>*>(smem);
  R* sc = reinterpret_cast<R*>(sp + kStage);                           // kStage x kMaxRhs complex
  double* red = reinterpret_cast<double*>(sc + 2 * kStage * kMaxRhs);  // blockDim x 2 kMaxDens
  const R isB = rcp(side_of(a, B));
  const int nsplit = (cnt > 0 && 2 * cnt <= (int)blockDim.x) ? (int)blockDim.x / cnt : 1;
  const int span = nsplit > 1 ? cnt : (int)blockDim.x;
  const int part = threadIdx.x / span, tj = threadIdx.x % span;
  for (int j0 = 0; j0 < cnt; j0 += span) {
    const int j = j0 + tj;
    const bool act = j < cnt && part < nsplit;
    Cx<R> u[kMaxDens];
#pragma unroll
    for (int d = 0; d < kMaxDens; ++d) u[d] = {(R)0, (R)0};
    Pos<R> tp{};
    if (act) {
      tp = pt_pos(a, s0 + j);
      const Cx<R> rho = cscale(vec(tp), isB);
#pragma unroll
      for (int d = 0; d < kMaxDens; ++d) {
        if (d < nq && d % nsplit == part) {
          const R* LA = a.local + 2 * (size_t)p * (3 * d + nch * (size_t)B);
          const R* LB = LA + 2 * (size_t)p;
          const R* LG = LB + 2 * (size_t)p;
          Cx<R> hA = ld_c(LA, p - 1), dA = {(R)0, (R)0};
          Cx<R> hB = ld_c(LB, p - 1);
          Cx<R> hG = ld_c(LG, p - 1), dG = {(R)0, (R)0};
          for (int l = p - 2; l >= 0; --l) {
            dA = cadd(cmul(dA, rho), hA);
            hA = cadd(cmul(hA, rho), ld_c(LA, l));
            hB = cadd(cmul(hB, rho), ld_c(LB, l));
            dG = cadd(cmul(dG, rho), hG);
            hG = cadd(cmul(hG, rho), ld_c(LG, l));
          }
          const Cx<R> c3 = cadd(cmul(cconj(rho), dA), cscale(dG, isB));
          u[d] = cadd(u[d], csub(cadd(hA, cconj(hB)), cconj(c3)));
        }
      }
      for (int wi = a.w_off[B]; wi < a.w_off[B + 1]; ++wi) {
        const int C = a.w_idx[wi];
        const Cx<R> w = cadd(vec(tp), box_off(a, C, B));  // z - c_C
        const Cx<R> iw = cinv(w);
        const Cx<R> t = cscale(iw, side_of(a, C));
        const Cx<R> iw2 = cmul(iw, iw);
#pragma unroll
        for (int d = 0; d < kMaxDens; ++d) {
          if (d < nq && d % nsplit == part) {
            const R* MA = a.mpole + 2 * (size_t)p * (3 * d + nch * (size_t)C);
            const R* MB = MA + 2 * (size_t)p;
            const R* ME = MB + 2 * (size_t)p;
            const R kp = to_r<R>((double)p);
            Cx<R> hA = ld_c(MA, p - 1), kA = cscale(ld_c(MA, p - 1), kp);
            Cx<R> hB = ld_c(MB, p - 1), kE = cscale(ld_c(ME, p - 1), kp);
            for (int k = p - 2; k >= 0; --k) {
              const R k1 = to_r<R>((double)(k + 1));
              hA = cadd(cmul(hA, t), ld_c(MA, k));
              kA = cadd(cmul(kA, t), cscale(ld_c(MA, k), k1));
              hB = cadd(cmul(hB, t), ld_c(MB, k));
              kE = cadd(cmul(kE, t), cscale(ld_c(ME, k), k1));
            }
            // S = iw h, S' = -iw^2 sum (k+1) M_k t^k
            const Cx<R> SA = cmul(iw, hA), SB = cmul(iw, hB);
            const Cx<R> dSA = cmul(iw2, kA), dSE = cmul(iw2, kE);  // -S'
            // conj(S_E' - conj(w) S_A') = conj(conj(w) dSA - dSE)
            const Cx<R> c3 = csub(cmul(cconj(w), dSA), dSE);
            u[d] = cadd(u[d], cadd(cadd(SA, cconj(SB)), cconj(c3)));
          }
        }
      }
    }
    for (int ui = a.u_off[B]; ui < a.u_off[B + 1]; ++ui) {
      const int D = a.u_idx[ui];
      const int d0 = a.pstart[D], dcnt = a.pcount[D];
      const auto offD = p2p_off(a, B, D);
      for (int i0 = 0; i0 < dcnt; i0 += kStage) {
        const int ic = dcnt - i0 < kStage ? dcnt - i0 : kStage;
        __syncthreads();
        for (int e = threadIdx.x; e < ic; e += blockDim.x) sp[e] = pt_pos(a, d0 + i0 + e);
        for (int e = threadIdx.x; e < ic * nch; e += blockDim.x) {
          const int i = e % ic, q = e / ic;
          const size_t src = d0 + i0 + i + (size_t)a.npts * q;
          sc[2 * (i + kStage * q)] = a.charge[2 * src];
          sc[2 * (i + kStage * q) + 1] = a.charge[2 * src + 1];
        }
        __syncthreads();
        if (act) {
          for (int i = part; i < ic; i += nsplit) {
            if (d0 + i0 + i == s0 + j) continue;  // self
            const Cx<R> tau = diff(tp, sp[i], offD);
            const Cx<R> iv = cinv(tau);
            const Cx<R> q2 = cmul(cconj(tau), cmul(iv, iv));  // conj(tau) / tau^2
#pragma unroll
            for (int d = 0; d < kMaxDens; ++d) {
              if (d < nq) {
                const Cx<R> av = {sc[2 * (i + kStage * 3 * d)], sc[2 * (i + kStage * 3 * d) + 1]};
                const R bv = sc[2 * (i + kStage * (3 * d + 1))];
                u[d] = cadd(u[d], cadd(cadd(cmul(av, iv), cscale(cconj(iv), bv)),
                                       cconj(cmul(av, q2))));
              }
            }
          }
        }
      }
    }
    double tot[2 * kMaxDens];
#pragma unroll
    for (int d = 0; d < kMaxDens; ++d) {
      tot[2 * d] = (double)u[d].re;
      tot[2 * d + 1] = (double)u[d].im;
    }
    if (nsplit > 1) {
      __syncthreads();
      if (act)
#pragma unroll
        for (int q = 0; q < 2 * kMaxDens; ++q) red[threadIdx.x * 2 * kMaxDens + q] = tot[q];
      __syncthreads();
      if (act && part == 0)
        for (int t = 1; t < nsplit; ++t)
#pragma unroll
          for (int q = 0; q < 2 * kMaxDens; ++q) tot[q] += red[(t * span + tj) * 2 * kMaxDens + q];
    }
    if (act && part == 0) {
      const int pt = a.slot_pt[s0 + j];
      const double nx = g.nx[pt], ny = g.ny[pt], tx = -ny, ty = nx;
      const double pot = -0.5 * g.kap[pt] * g.w[pt] * (1.0 / CUDART_PI);
      const size_t D = 2 * (size_t)a.npts;
#pragma unroll
      for (int d = 0; d < kMaxDens; ++d) {
        if (d < nq) {
          const size_t o = 2 * (size_t)pt + D * d;
          const double mx = mu[o], my = mu[o + 1];
          const double tm = pot * (tx * mx + ty * my);
          const double vx = yb * (-0.5 * mx + tm * tx + nx * r1[d] + tot[2 * d]);
          const double vy = yb * (-0.5 * my + tm * ty + ny * r1[d] + tot[2 * d + 1]);
          y[o] = ya == 0.0 ? vx : ya * y[o] + vx;
          y[o + 1] = ya == 0.0 ? vy : ya * y[o + 1] + vy;
        }
      }
    }
  }
}

// Grid of the near-field kernel on the side stream: half the CTAs that fit
// on the GPU at once (at most one per leaf), so that the tree passes'
// launches find free slots beside it instead of waiting for its CTAs to
// retire.
template <class R>
unsigned near_grid(unsigned nleaves) {
  static unsigned cap = 0;
  if (cap == 0) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, eval_warp_kernel<R, kEvalNear>,
                                                  32 * kEvalWarps, 0);
    cap = (unsigned)std::max(1, sms * std::max(1, per / 2));
  }
  return std::min(nleaves, cap);
}

template <class R>
cudaError_t apply_t(FmmPlan& f, int mode, const Geo<double>& geo, const double* mu, int nrhs,
                    double* y, double ya, double yb, cudaStream_t st) {
  constexpr bool f32 = std::is_same<R, float>::value;
  const int p = f32 ? f.p32 : f.p;
  const int npts = f.npts, nb = f.nbox;
  if (p < 2 || p * kMaxRhs > 4 * kFmmThreads || (f32 && p > f.p32_tab))
    return cudaErrorInvalidValue;
  set_smem_once<p2m_kernel<R>>();
  set_smem_once<m2m_kernel<R>>();
  set_smem_once<m2l_kernel<R>>();
  set_smem_once<l2l_kernel<R>>();
  const int pmax = f.p > f.p32 ? f.p : f.p32;
  cudaError_t e;
  if ((e = f.charge.ensure(2 * (size_t)npts * kMaxRhs)) != cudaSuccess) return e;
  // (sized in doubles: holds kSrcStride values of R <= 8 bytes per slot)
  if ((e = f.src.ensure((size_t)npts * kSrcStride)) != cudaSuccess) return e;
  if ((e = f.mpole.ensure(2 * (size_t)pmax * kMaxRhs * nb)) != cudaSuccess) return e;
  if ((e = f.local.ensure(2 * (size_t)pmax * kMaxRhs * nb)) != cudaSuccess) return e;
  if ((e = f.r1.ensure(kMaxRhs)) != cudaSuccess) return e;
  if (mode != 2) {
    if ((e = f.nearsum.ensure((size_t)npts * kMaxRhs)) != cudaSuccess) return e;
    if (f.nearq.st == nullptr) {
      int lo = 0, hi = 0;
      if ((e = cudaDeviceGetStreamPriorityRange(&lo, &hi)) != cudaSuccess) return e;
      // (lo is the numerically greatest value: the lowest priority)
      if ((e = cudaStreamCreateWithPriority(&f.nearq.st, cudaStreamNonBlocking, lo)) != cudaSuccess)
        return e;
      if ((e = cudaEventCreateWithFlags(&f.nearq.charges, cudaEventDisableTiming)) != cudaSuccess)
        return e;
      if ((e = cudaEventCreateWithFlags(&f.nearq.near, cudaEventDisableTiming)) != cudaSuccess)
        return e;
      if ((e = cudaEventCreateWithFlags(&f.nearq.mpole, cudaEventDisableTiming)) != cudaSuccess)
        return e;
    }
  }
  FmmArgs<R> a{};
  a.cx = f.cx.p;
  a.cy = f.cy.p;
  a.side = f.side.p;
  a.rx = f.rx.p;
  a.ry = f.ry.p;
  a.rxh = f.rxh.p;
  a.rxl = f.rxl.p;
  a.ryh = f.ryh.p;
  a.ryl = f.ryl.p;
  a.bs = f32 ? 2 * f.p32_tab : 2 * f.p;
  if constexpr (f32) a.binom = f.binom32.p;
  else if constexpr (std::is_same<R, DF>::value) a.binom = reinterpret_cast<const DF*>(f.binom_df.p);
  else a.binom = f.binom.p;
  a.pstart = f.pstart.p;
  a.pcount = f.pcount.p;
  a.parent = f.parent.p;
  a.slot_pt = f.slot_pt.p;
  a.children = f.children.p;
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
  a.mode = mode;
  R* charge = reinterpret_cast<R*>(f.charge.p);
  a.charge = charge;
  R* src = reinterpret_cast<R*>(f.src.p);
  a.src = src;
  a.mpole = reinterpret_cast<R*>(f.mpole.p);
  a.local = reinterpret_cast<R*>(f.local.p);
  const unsigned nleaves = (unsigned)f.leaves_h.size();
  // densities per pass: one channel each (Laplace, Neumann) or three (Stokes)
  const int per = mode == 2 ? kMaxDens : kMaxRhs;
  const size_t dcol = (size_t)npts * (mode == 2 ? 2 : 1);
  for (int q0 = 0; q0 < nrhs; q0 += per) {
    const int nq = nrhs - q0 < per ? nrhs - q0 : per;
    const int nch = mode == 2 ? 3 * nq : nq;
    a.nrhs = nch;
    const double* muq = mu + dcol * q0;
    double* yq = y + dcol * q0;
    const size_t tot = (size_t)npts * nq;
    const unsigned cg = (unsigned)((tot + 255) / 256);
    if (mode == 0) {
      charges_kernel<R><<<cg, 256, 0, st>>>(geo, f.slot_pt.p, npts, muq, nq, charge, src);
    } else if (mode == 1) {
      neumann_charges_kernel<R><<<cg, 256, 0, st>>>(geo, f.slot_pt.p, npts, muq, nq, charge,
                                                    src);
    } else {
      stokes_charges_kernel<R><<<cg, 256, 0, st>>>(geo, f.slot_pt.p, f.rx.p, f.ry.p, npts, muq,
                                                   nq, charge);
    }
    if (mode != 0) rank1_kernel<<<nq, 1024, 0, st>>>(geo, npts, muq, mode, f.r1.p);
    // the near field on the side stream (Laplace, Neumann), once the charges
    // kernel's source data are written
    const bool split = mode != 2 && nleaves > 0 && f.nearq.st != nullptr;
    if (split) {
      a.boxes = f.leaves.p;  // the kernel's boxes are the leaves
      if ((e = cudaEventRecord(f.nearq.charges, st)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(f.nearq.st, f.nearq.charges, 0)) != cudaSuccess) return e;
      eval_warp_kernel<R, kEvalNear><<<near_grid<R>(nleaves), 32 * kEvalWarps, 0, f.nearq.st>>>(
          a, geo, muq, yq, ya, yb, (const double*)f.r1.p, f.nearsum.p, (int)nleaves);
      if (!std::is_same<R, DF>::value &&
          (e = cudaEventRecord(f.nearq.near, f.nearq.st)) != cudaSuccess)
        return e;
    }
    // upward pass
    a.boxes = f.leaves.p;
    if (nleaves)
      launch_pdl(p2m_kernel<R>, dim3(nleaves), dim3(kFmmThreads),
                 sizeof(Cx<R>) * kStage * (size_t)p, st, a);
    // levels 0 and 1 have no V, W or X partners: their multipoles are unused
    for (int lv = f.nlevels - 2; lv >= 2; --lv) {
      const int cnt = f.level_off[lv + 1] - f.level_off[lv];
      if (!cnt) continue;
      a.boxes = f.lvl_boxes.p + f.level_off[lv];
      launch_pdl(m2m_kernel<R>, dim3(cnt), dim3(kFmmThreads),
                 sizeof(Cx<R>) * (8 * (size_t)p + 4 * (size_t)p * nch + 4), st, a);
    }
    const bool wsplit = split && std::is_same<R, DF>::value;
    if (wsplit) {
      // M2P over the W lists on the side stream, once the multipoles are done
      if ((e = cudaEventRecord(f.nearq.mpole, st)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(f.nearq.st, f.nearq.mpole, 0)) != cudaSuccess) return e;
      a.boxes = f.leaves.p;
      eval_warp_kernel<R, kEvalW><<<near_grid<R>(nleaves), 32 * kEvalWarps, 0, f.nearq.st>>>(
          a, geo, muq, yq, ya, yb, (const double*)f.r1.p, f.nearsum.p, (int)nleaves);
      if ((e = cudaEventRecord(f.nearq.near, f.nearq.st)) != cudaSuccess) return e;
    }
    // interactions and downward pass
    if ((e = cudaMemsetAsync(f.local.p, 0, 2 * sizeof(R) * (size_t)p * nch * nb, st)) !=
        cudaSuccess)
      return e;
    if (!f.m2l_boxes_h.empty()) {
      a.boxes = f.m2l_boxes.p;
      m2l_kernel<R><<<(unsigned)f.m2l_boxes_h.size(), kFmmThreads,
                      sizeof(Cx<R>) * ((size_t)p * nch + p + kStage * (size_t)p + kStage + 1),
                      st>>>(a);
    }
    // locals of levels <= 2 come only from M2L (level 0/1 locals are zero)
    for (int lv = 3; lv < f.nlevels; ++lv) {
      const int cnt = f.level_off[lv + 1] - f.level_off[lv];
      if (!cnt) continue;
      a.boxes = f.lvl_boxes.p + f.level_off[lv];
      launch_pdl(l2l_kernel<R>, dim3(cnt), dim3(kFmmThreads),
                 sizeof(Cx<R>) * (2 * (size_t)p + (size_t)p * nch), st, a);
    }
    a.boxes = f.leaves.p;
    const size_t esm = sizeof(Pos<R>) * kStage + sizeof(Cx<R>) * kStage * kMaxRhs +
                       sizeof(double) * kEvalThreads * kMaxRhs;
    if (nleaves && mode == 2) {
      stokes_eval_kernel<R><<<nleaves, kEvalThreads, esm, st>>>(a, geo, muq, yq, ya, yb, f.r1.p);
    } else if (split) {
      // the far field, after the near field on the side stream
      if ((e = cudaStreamWaitEvent(st, f.nearq.near, 0)) != cudaSuccess) return e;
      if (wsplit)
        eval_warp_kernel<R, kEvalFar><<<nleaves, 32 * kEvalWarps, 0, st>>>(
            a, geo, muq, yq, ya, yb, (const double*)f.r1.p, f.nearsum.p, (int)nleaves);
      else
        eval_warp_kernel<R, kEvalFarW><<<nleaves, 32 * kEvalWarps, 0, st>>>(
            a, geo, muq, yq, ya, yb, (const double*)f.r1.p, f.nearsum.p, (int)nleaves);
    } else if (nleaves) {
      launch_pdl(eval_warp_kernel<R, kEvalAll>, dim3(nleaves), dim3(32 * kEvalWarps), 0, st, a,
                 geo, muq, yq, ya, yb, (const double*)f.r1.p, (double*)nullptr, (int)nleaves);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

int fmm_launches(const FmmPlan& f, int pde, int nrhs) {
  const int per = pde == 2 ? kMaxDens : kMaxRhs;
  const int passes = (nrhs + per - 1) / per;
  int k = 1 + (pde != 0) + (f.leaves_h.empty() ? 0 : 2) + (f.m2l_boxes_h.empty() ? 0 : 1);
  for (int lv = f.nlevels - 2; lv >= 2; --lv) k += f.level_off[lv + 1] > f.level_off[lv];
  for (int lv = 3; lv < f.nlevels; ++lv) k += f.level_off[lv + 1] > f.level_off[lv];
  return passes * k;
}

cudaError_t fmm_apply(FmmPlan& f, int pde, const Geo<double>& geo, const double* mu, int nrhs,
                      double* y, double ya, double yb, int arith, cudaStream_t st) {
  if (!f.built || pde < 0 || pde > 2) return cudaErrorInvalidValue;
  switch (arith) {
    case kFmmF64: return apply_t<double>(f, pde, geo, mu, nrhs, y, ya, yb, st);
    case kFmmF32: return apply_t<float>(f, pde, geo, mu, nrhs, y, ya, yb, st);
    case kFmmDF: return apply_t<DF>(f, pde, geo, mu, nrhs, y, ya, yb, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace rskel
