/*
 * lgb_eval.cuh -- partition-of-unity RBF evaluation at particles.
 *
 * Replaces RBFInterpolation -> PointwiseInterpolation_{AVX512,AVX256,Scalar}
 * (src/interpolation/interpolation.c:39-154, 178-272; interpolation_avx512.c:121-291) and the PU
 * weights of SwarmInterpSetWeights (src/swarm/swarm_interp.c:283-396, weights_avx.c:97-243):
 *
 *   v_f(x_p) = sum_{k in corners(cell p)} w_k(x_p) * sum_{j in patch k} phi(|x_p - x_j|, eps_r) X_k[j, f]
 *   w_k(x)   = phiW(|x - c_k|, eps_w) / sum_{all nodes n} phiW(|x - c_n|, eps_w)     (Wendland C2)
 *
 * This file holds the gather evaluation (the FP64 path, and FP32 where no record blocks exist) and
 * the pieces both evaluations share; the FP32 evaluation from TMA-streamed record blocks, the hot
 * kernel of the FP32 path, is k_eval_rec in lgb_evalrec.cuh.
 *
 * GB300 design.  Particles are binned by cell every stage; one CTA evaluates one work unit of up to
 * chunk_cap particles of one cell.  The CTA walks the 3^dim neighbour cells of its cell in the
 * reference's neighbour order, staging for each neighbour cell a record per data point
 * {x, y, z, pad, X_k[j, f] for every corner patch k of the particle's cell that contains the
 * neighbour cell} in shared memory (a fixed budget, refilled in rounds when the block does not
 * fit).  Every thread then reads the same record (broadcast, no bank conflicts): phi is computed
 * once per (particle, data point) and feeds the accumulators of every patch that holds the point,
 * so the per-patch sums run in the reference's patch order (cells ascending, points ascending).
 * Which patches a neighbour offset touches is a compile-time mask, so the accumulators stay in
 * registers.  The PU weights need only the support nodes (<= (2*wr+2)^dim candidates): the
 * reference's sum over all nodes adds exact zeros outside the support.
 *
 * Precision.  The FP64 variant follows the reference arithmetic (absolute coordinates, FP64 phi,
 * w_k = phiW_k / sum, v += I_k * w_k).  The FP32 variant computes coordinates relative to the cell
 * origin (so distances keep their relative precision), phi and the per-patch sums in FP32, the
 * PU-weighted sum sum_k phiW_k * I_k with an error-free compensated accumulation (TwoSum/TwoProd
 * into a float pair), and the weight normalisation in FP64.
 *
 * Roofline: FP32 (or FP64) pipe bound; per particle ~B_c*(10 + k_phi) + 2*F*sum_k m_k flops against
 * ~(28 + 8F) bytes of particle traffic, with the block data reused by every particle of the cell.
 */
#pragma once
#include <type_traits>
#include "lgb_common.cuh"

struct EvalParams {
  lgb_geom g;
  const int *cstart;
  const float *xr32;      /* [nd*4] cell-relative f32 coordinates, cell order        */
  const double *xs64;     /* [nd*dim] f64 coordinates, cell order                    */
  const float *c32;
  const double *c64;
  const long long *coff;
  const int *slot;
  const int *setup;
  int F, f0;
  const int *pstart, *plist, *chunk_start;
  const double *xp;
  double *out;
  int out_stride;
  lgb_ctrl *ctrl;
  int budget;             /* staging budget, elements of the compute type (per buffer) */
  int chunk_cap;          /* particles per work unit (blockDim.x * R)     */
  float *rec32;           /* precomputed FP32 record blocks (streamed by k_eval_rec) */
  const long long *rec_off;
  int poll_limit;         /* polls of a bounded mbarrier wait before it gives up          */
  int withhold_copies;    /* test hook: arm the staging barriers but issue no copy         */
  unsigned char *cdirty;  /* cells whose record blocks must be rebuilt (set by the work-list compaction) */
};

enum { KER_GENERIC = 0, KER_C2 = 1, KER_GAUSS = 2 };

template <int DIM> struct EGeo {
  static constexpr int NOFF = (DIM == 3) ? 27 : 9;
  static constexpr int NEN = 1 << DIM;
};

__host__ __device__ constexpr int eoff_a(int o) { return o % 3 - 1; }
__host__ __device__ constexpr int eoff_b(int o) { return (o / 3) % 3 - 1; }
__host__ __device__ constexpr int eoff_e(int dim, int o) { return dim == 3 ? o / 9 - 1 : 0; }
__host__ __device__ constexpr int ecorner_ox(int k) { return ((k & 3) == 1 || (k & 3) == 2) ? 1 : 0; }
__host__ __device__ constexpr int ecorner_oy(int k) { return ((k & 3) >= 2) ? 1 : 0; }
__host__ __device__ constexpr int ecorner_oz(int dim, int k) { return dim == 3 ? (k >> 2) : 0; }

/* Corner patches of the particle's cell that contain neighbour cell `o`. */
__host__ __device__ constexpr int einv_mask(int dim, int o)
{
  int m = 0;
  for (int k = 0; k < (1 << dim); k++) {
    int a = eoff_a(o), b = eoff_b(o), e = eoff_e(dim, o);
    int ox = ecorner_ox(k), oy = ecorner_oy(k), oz = ecorner_oz(dim, k);
    bool in = (a == ox - 1 || a == ox) && (b == oy - 1 || b == oy) && (dim == 2 || e == oz - 1 || e == oz);
    if (in) m |= 1 << k;
  }
  return m;
}
__host__ __device__ constexpr int epopc(int m) { return m == 0 ? 0 : (m & 1) + epopc(m >> 1); }
/* Slot of neighbour cell o inside the patch of corner k (ascending cell order of the patch). */
__host__ __device__ constexpr int eslot(int dim, int k, int o)
{
  return (eoff_a(o) - ecorner_ox(k) + 1) + 2 * (eoff_b(o) - ecorner_oy(k) + 1) +
         (dim == 3 ? 4 * (eoff_e(dim, o) - ecorner_oz(dim, k) + 1) : 0);
}
/* Record length (elements) for a neighbour offset: 4 coordinates + ninv*FP coefficients, padded
   to a 16-byte multiple. */
template <typename Real> __host__ __device__ constexpr int erec(int ninv, int fp)
{
  return sizeof(Real) == 4 ? LGB_REC32_LEN(ninv, fp) : ((4 + ninv * fp + 1) / 2) * 2;
}
/* Record layout: coordinate d at rec[d * EXS], coefficient (field f, patch j) at
   rec[EHEAD + (f * ninv + j) * EDUP] (FP64 records: {x, y, z, 0} and single coefficients). */
template <typename Real> __host__ __device__ constexpr int ehead() { return sizeof(Real) == 4 ? LGB_REC32_HEAD : 4; }
template <typename Real> __host__ __device__ constexpr int edup() { return sizeof(Real) == 4 ? LGB_REC32_DUP : 1; }
template <typename Real> __host__ __device__ constexpr int exs() { return sizeof(Real) == 4 ? 2 : 1; }

template <typename Real, int KER>
__device__ __forceinline__ Real eval_phi(Real d2, Real eps, Real ga, int kernel)
{
  if constexpr (sizeof(Real) == 4 && KER == KER_C2) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(d2)); /* one MUFU op; exact at 0 */
    float u = fmaxf(1.0f - eps * r, 0.0f);
    float u2 = u * u;
    return (u2 * u2) * (5.0f - 4.0f * u);
  } else if constexpr (sizeof(Real) == 4 && KER == KER_GAUSS) {
    return exp2f(ga * d2);
  } else {
    return lgb_phi<Real>(kernel, sqrt(d2), eps);
  }
}

#define LGB_PRAGMA(x) _Pragma(#x)
#define LGB_UNROLL(n) LGB_PRAGMA(unroll n)
#ifndef LGB_X2_UNROLL
#define LGB_X2_UNROLL 2 /* points of a segment in flight per thread in the packed FP32 loop */
#endif

/* ---- packed FP32 pairs (PTX .f32x2, sm_100 and later): one instruction applies the IEEE
   single-precision operation to both halves of a 64-bit register pair ---- */
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 x2_pack(float a, float b)
{
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void x2_unpack(f32x2 v, float &a, float &b)
{
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c)
{
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f32x2 x2_mul(f32x2 a, f32x2 b)
{
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_add(f32x2 a, f32x2 b)
{
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_sub(f32x2 a, f32x2 b)
{
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

/* index of the j-th set bit of mask (the corner of the j-th involved patch) */
__host__ __device__ constexpr int ekj(int mask, int j)
{
  for (int k = 0; k < 8; k++)
    if ((mask >> k) & 1) {
      if (j == 0) return k;
      --j;
    }
  return 0;
}

/* FP32 segment with two particles per thread on packed pairs: the distances and the Wendland C2
   polynomial run on (particle 0, particle 1) pairs against the record's duplicated coordinates.
   With duplicated coefficients (LGB_REC32_DUP == 2) the sums also run on particle pairs; otherwise
   on (patch 2i, patch 2i+1) pairs of one field.  Each lane performs the same IEEE operations in the
   same order as the scalar form, so the results are identical to it.  Partial sums of the segment
   go to the running sums at the end (blocked accumulation). */
template <int DIM, int FP, int KER, int NI>
__device__ __forceinline__ void eval_segment_x2(const float *__restrict__ rec, int n, const float (&px)[2][3], float eps,
                                                float ga, float *__restrict__ run, int mask)
{
  constexpr int NEN = EGeo<DIM>::NEN;
  constexpr int H = LGB_REC32_HEAD;
  constexpr int S = erec<float>(NI, FP);
  constexpr int NV = S / 4;
  constexpr bool DUP = (LGB_REC32_DUP == 2);
  constexpr int NP = DUP ? NI : NI / 2;     /* accumulator pairs per field */
  constexpr bool ODD = !DUP && (NI & 1);    /* one unpaired patch (NI == 1) */
  const f32x2 pxx = x2_pack(px[0][0], px[1][0]), pyy = x2_pack(px[0][1], px[1][1]);
  const f32x2 pzz = x2_pack(px[0][2], px[1][2]);
  const f32x2 neps = x2_pack(-eps, -eps), one = x2_pack(1.f, 1.f), m4 = x2_pack(-4.f, -4.f), five = x2_pack(5.f, 5.f);
  f32x2 ap[FP][NP > 0 ? NP : 1];    /* DUP: lanes = particles; else lanes = patches, particle 0 */
  f32x2 bp[FP][(!DUP && NP > 0) ? NP : 1]; /* !DUP: particle 1 */
  float as[2][FP];
#pragma unroll
  for (int f = 0; f < FP; f++) {
    as[0][f] = 0.f;
    as[1][f] = 0.f;
#pragma unroll
    for (int q = 0; q < (NP > 0 ? NP : 1); q++) ap[f][q] = 0ull;
#pragma unroll
    for (int q = 0; q < ((!DUP && NP > 0) ? NP : 1); q++) bp[f][q] = 0ull;
  }
  LGB_UNROLL(LGB_X2_UNROLL)
  for (int p = 0; p < n; ++p) {
    float v[S];
    const float4 *rv = reinterpret_cast<const float4 *>(rec + (size_t)p * S);
#pragma unroll
    for (int q = 0; q < NV; q++) {
      const float4 t = rv[q];
      v[4 * q + 0] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
    }
    const f32x2 dx = x2_sub(pxx, x2_pack(v[0], v[1]));
    const f32x2 dy = x2_sub(pyy, x2_pack(v[2], v[3]));
    f32x2 d2;
    if constexpr (DIM == 3) {
      const f32x2 dz = x2_sub(pzz, x2_pack(v[4], v[5]));
      d2 = x2_fma(dx, dx, x2_fma(dy, dy, x2_mul(dz, dz)));
    } else {
      d2 = x2_fma(dx, dx, x2_mul(dy, dy));
    }
    float d2a, d2b;
    x2_unpack(d2, d2a, d2b);
    f32x2 ph;
    if constexpr (KER == KER_C2) {
      float ra, rb;
      asm("sqrt.approx.f32 %0, %1;" : "=f"(ra) : "f"(d2a));
      asm("sqrt.approx.f32 %0, %1;" : "=f"(rb) : "f"(d2b));
      float ua, ub;
      x2_unpack(x2_fma(x2_pack(ra, rb), neps, one), ua, ub); /* 1 - eps*r */
      const f32x2 u = x2_pack(fmaxf(ua, 0.f), fmaxf(ub, 0.f));
      const f32x2 u2 = x2_mul(u, u);
      ph = x2_mul(x2_mul(u2, u2), x2_fma(u, m4, five));
    } else {
      ph = x2_pack(exp2f(ga * d2a), exp2f(ga * d2b));
    }
    if constexpr (DUP) {
#pragma unroll
      for (int f = 0; f < FP; f++)
#pragma unroll
        for (int j = 0; j < NI; j++)
          ap[f][j] = x2_fma(ph, x2_pack(v[H + 2 * (f * NI + j)], v[H + 2 * (f * NI + j) + 1]), ap[f][j]);
    } else {
      float pa, pb;
      x2_unpack(ph, pa, pb);
      const f32x2 PA = x2_pack(pa, pa), PB = x2_pack(pb, pb);
#pragma unroll
      for (int f = 0; f < FP; f++) {
#pragma unroll
        for (int q = 0; q < NP; q++) {
          const f32x2 c = x2_pack(v[H + f * NI + 2 * q], v[H + f * NI + 2 * q + 1]);
          ap[f][q] = x2_fma(PA, c, ap[f][q]);
          bp[f][q] = x2_fma(PB, c, bp[f][q]);
        }
        if constexpr (ODD) {
          const float c = v[H + f * NI + NI - 1];
          as[0][f] = fmaf(pa, c, as[0][f]);
          as[1][f] = fmaf(pb, c, as[1][f]);
        }
      }
    }
  }
  /* corners of the involved patches, in record order (ascending corner index) */
  int kj[NI];
  unsigned m = (unsigned)mask;
#pragma unroll
  for (int j = 0; j < NI; j++) {
    kj[j] = __ffs(m) - 1;
    m &= m - 1;
  }
#pragma unroll
  for (int f = 0; f < FP; f++) {
    if constexpr (DUP) {
#pragma unroll
      for (int j = 0; j < NI; j++) {
        float a, b;
        x2_unpack(ap[f][j], a, b);
        run[(0 * NEN + kj[j]) * FP + f] += a;
        run[(1 * NEN + kj[j]) * FP + f] += b;
      }
    } else {
#pragma unroll
      for (int q = 0; q < NP; q++) {
        float lo, hi;
        x2_unpack(ap[f][q], lo, hi);
        run[(0 * NEN + kj[2 * q]) * FP + f] += lo;
        run[(0 * NEN + kj[2 * q + 1]) * FP + f] += hi;
        x2_unpack(bp[f][q], lo, hi);
        run[(1 * NEN + kj[2 * q]) * FP + f] += lo;
        run[(1 * NEN + kj[2 * q + 1]) * FP + f] += hi;
      }
      if constexpr (ODD) {
        run[(0 * NEN + kj[NI - 1]) * FP + f] += as[0][f];
        run[(1 * NEN + kj[NI - 1]) * FP + f] += as[1][f];
      }
    }
  }
}

/* Accumulate one staged segment of neighbour offset O. */
template <typename Real, int DIM, int FP, int R, int KER, int O>
__device__ __forceinline__ void eval_segment(const Real *__restrict__ rec, int n, const Real (&px)[R][3],
                                             Real (&acc)[R][EGeo<DIM>::NEN][FP], Real eps, Real ga, int kernel,
                                             float *__restrict__ run, int rstride)
{
  constexpr int NEN = EGeo<DIM>::NEN;
  constexpr int MASK = einv_mask(DIM, O);
  constexpr int NI = epopc(MASK);
  constexpr int S = erec<Real>(NI, FP);
  using V = typename std::conditional<sizeof(Real) == 4, float4, double2>::type;
  constexpr int VW = sizeof(V) / sizeof(Real);
  constexpr int NV = S / VW;
#pragma unroll 1
  for (int p = 0; p < n; ++p) {
    Real v[S];
    const V *rv = reinterpret_cast<const V *>(rec + (size_t)p * S);
#pragma unroll
    for (int q = 0; q < NV; q++) {
      V t = rv[q];
      if constexpr (VW == 4) {
        v[4 * q + 0] = ((const float *)&t)[0]; v[4 * q + 1] = ((const float *)&t)[1];
        v[4 * q + 2] = ((const float *)&t)[2]; v[4 * q + 3] = ((const float *)&t)[3];
      } else {
        v[2 * q + 0] = ((const double *)&t)[0]; v[2 * q + 1] = ((const double *)&t)[1];
      }
    }
    Real phi[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      Real dx = px[r][0] - v[0], dy = px[r][1] - v[exs<Real>()], d2;
      if constexpr (DIM == 3) {
        Real dz = px[r][2] - v[2 * exs<Real>()];
        d2 = fma(dx, dx, fma(dy, dy, dz * dz));
      } else {
        d2 = fma(dx, dx, dy * dy);
      }
      phi[r] = eval_phi<Real, KER>(d2, eps, ga, kernel);
    }
    int j = 0;
#pragma unroll
    for (int k = 0; k < NEN; k++) {
      if ((MASK >> k) & 1) {
#pragma unroll
        for (int f = 0; f < FP; f++) {
          Real cf = v[ehead<Real>() + (f * NI + j) * edup<Real>()];
#pragma unroll
          for (int r = 0; r < R; r++) acc[r][k][f] = fma(phi[r], cf, acc[r][k][f]);
        }
        j++;
      }
    }
  }
  if constexpr (sizeof(Real) == 4) {
    /* blocked summation: the segment's partial sums (one neighbour cell, <= budget points) go into
       per-thread running sums in shared memory, which bounds the FP32 accumulation error by the
       segment length instead of the patch size */
#pragma unroll
    for (int k = 0; k < NEN; k++) {
      if ((MASK >> k) & 1) {
#pragma unroll
        for (int f = 0; f < FP; f++)
#pragma unroll
          for (int r = 0; r < R; r++) {
            float *q = run + (r * NEN + k) * FP + f; /* this thread's slot block (compile-time offsets) */
            *q += acc[r][k][f];
            acc[r][k][f] = 0.f;
          }
      }
    }
  }
}

template <typename Real, int DIM, int FP, int R, int KER>
__device__ __forceinline__ void eval_dispatch(int o, const Real *rec, int n, const Real (&px)[R][3],
                                              Real (&acc)[R][EGeo<DIM>::NEN][FP], Real eps, Real ga, int kernel,
                                              float *run, int rstride)
{
#define EV_CASE(OO) case OO: eval_segment<Real, DIM, FP, R, KER, OO>(rec, n, px, acc, eps, ga, kernel, run, rstride); break;
  if constexpr (sizeof(Real) == 4 && R == 2 && (KER == KER_C2 || KER == KER_GAUSS)) {
    /* packed FP32 path: one code body per number of involved patches (1, 2, 4 or 8), the corner
       mapping is applied when the segment's sums are flushed */
    const float *rf = reinterpret_cast<const float *>(rec);
    const float(&pf)[2][3] = reinterpret_cast<const float(&)[2][3]>(px);
    const int mask = einv_mask(DIM, o);
    switch (epopc(mask)) {
    case 1: eval_segment_x2<DIM, FP, KER, 1>(rf, n, pf, (float)eps, (float)ga, run, mask); break;
    case 2: eval_segment_x2<DIM, FP, KER, 2>(rf, n, pf, (float)eps, (float)ga, run, mask); break;
    case 4: eval_segment_x2<DIM, FP, KER, 4>(rf, n, pf, (float)eps, (float)ga, run, mask); break;
    case 8: if constexpr (DIM == 3) eval_segment_x2<DIM, FP, KER, 8>(rf, n, pf, (float)eps, (float)ga, run, mask); break;
    default: break;
    }
  } else if constexpr (DIM == 3) {
    switch (o) {
      EV_CASE(0) EV_CASE(1) EV_CASE(2) EV_CASE(3) EV_CASE(4) EV_CASE(5) EV_CASE(6) EV_CASE(7) EV_CASE(8)
      EV_CASE(9) EV_CASE(10) EV_CASE(11) EV_CASE(12) EV_CASE(13) EV_CASE(14) EV_CASE(15) EV_CASE(16)
      EV_CASE(17) EV_CASE(18) EV_CASE(19) EV_CASE(20) EV_CASE(21) EV_CASE(22) EV_CASE(23) EV_CASE(24)
      EV_CASE(25) EV_CASE(26)
      default: break;
    }
  } else {
    switch (o) {
      EV_CASE(0) EV_CASE(1) EV_CASE(2) EV_CASE(3) EV_CASE(4) EV_CASE(5) EV_CASE(6) EV_CASE(7) EV_CASE(8)
      default: break;
    }
  }
#undef EV_CASE
}

/* Node-index range [lo, hi] along one axis that contains every node within the weight support of
   coordinate x. */
__device__ __forceinline__ void eval_node_range(double x, double O, double ih, int n, double rad, int &lo, int &hi)
{
  /* nodes i with |x - (O + i h)| < rad (ih = 1 / h); the 1e-6 margin (in node spacings) covers
     rounding, and a node at distance >= rad has phiW == 0 exactly, so the range is never too small */
  int a = (int)ceil((x - rad - O) * ih - 1e-6);
  int b = (int)floor((x + rad - O) * ih + 1e-6);
  lo = (a < 0) ? 0 : a;
  hi = (b > n - 1) ? n - 1 : b;
}

/* PU weights of one particle from the support nodes.  FP32: coordinates relative to the cell
   origin (node ci, cj, cl), compensated sum.  FP64: absolute node coordinates as in the
   reference.  pw[k] are the corner values phiW(|x - c_k|), den the sum over all nodes. */
template <typename Real, int DIM>
__device__ __forceinline__ void eval_weights(const lgb_geom &g, int ci, int cj, int cl, const double *x,
                                             const Real *xr, Real (&pw)[EGeo<DIM>::NEN], double &den, int &nsupp)
{
  constexpr int NEN = EGeo<DIM>::NEN;
  const double rad = g.rad_w;
  int ilo, ihi, jlo, jhi, klo = 0, khi = 0;
  eval_node_range(x[0], g.O[0], g.rh[0], g.n[0], rad, ilo, ihi);
  eval_node_range(x[1], g.O[1], g.rh[1], g.n[1], rad, jlo, jhi);
  if constexpr (DIM == 3) eval_node_range(x[2], g.O[2], g.rh[2], g.n[2], rad, klo, khi);
  nsupp = 0;
  if constexpr (sizeof(Real) == 4) {
    const float epsw = (float)g.eps_w, hf0 = (float)g.h[0], hf1 = (float)g.h[1], hf2 = (float)g.h[2];
    float shi = 0.f, slo = 0.f;
    for (int k = klo; k <= khi; k++) {
      const float dz = (DIM == 3) ? xr[2] - (float)(k - cl) * hf2 : 0.f;
      for (int j = jlo; j <= jhi; j++) {
        const float dy = xr[1] - (float)(j - cj) * hf1;
        for (int i = ilo; i <= ihi; i++) {
          const float dx = xr[0] - (float)(i - ci) * hf0;
          const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const float w = lgb_wendland_c2<float>(sqrtf(d2), epsw);
          nsupp += (w > 0.f);
          lgb_df_add(shi, slo, w);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NEN; q++) {
      float dx = xr[0] - ecorner_ox(q) * hf0, dy = xr[1] - ecorner_oy(q) * hf1;
      float dz = (DIM == 3) ? xr[2] - ecorner_oz(DIM, q) * hf2 : 0.f;
      pw[q] = lgb_wendland_c2<float>(sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))), epsw);
    }
    den = (double)shi + (double)slo;
  } else {
    double sum = 0.0;
    for (int k = klo; k <= khi; k++) {
      const double dz = (DIM == 3) ? x[2] - (g.O[2] + g.h[2] * k) : 0.0;
      for (int j = jlo; j <= jhi; j++) {
        const double dy = x[1] - (g.O[1] + g.h[1] * j);
        for (int i = ilo; i <= ihi; i++) {
          const double dx = x[0] - (g.O[0] + g.h[0] * i);
          const double d2 = (DIM == 3) ? fma(dx, dx, fma(dy, dy, dz * dz)) : fma(dx, dx, dy * dy);
          const double w = lgb_wendland_c2<double>(sqrt(d2), g.eps_w);
          nsupp += (w > 0.0);
          sum += w;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NEN; q++) {
      const double dx = x[0] - (g.O[0] + g.h[0] * (ci + ecorner_ox(q)));
      const double dy = x[1] - (g.O[1] + g.h[1] * (cj + ecorner_oy(q)));
      const double dz = (DIM == 3) ? x[2] - (g.O[2] + g.h[2] * (cl + ecorner_oz(DIM, q))) : 0.0;
      const double d2 = (DIM == 3) ? fma(dx, dx, fma(dy, dy, dz * dz)) : fma(dx, dx, dy * dy);
      pw[q] = (Real)lgb_wendland_c2<double>(sqrt(d2), g.eps_w);
    }
    den = sum;
  }
}

/* One record of the staged block: coordinates of data point `sidx` (neighbour offset o, position
   pp inside its cell) relative to the origin of cell (ci, cj, cl), then the FP coefficients of every
   corner patch k of that cell containing the neighbour cell (zeros for patches not set up),
   zero-padded to the record length. */
template <typename Real, int DIM, int FP>
__device__ __forceinline__ void write_record(const EvalParams &P, int o, int pp, int sidx, const int *node,
                                             const int *setup, Real *rec)
{
  constexpr int NEN = EGeo<DIM>::NEN;
  const int mask = einv_mask(DIM, o);
  const int S = erec<Real>(epopc(mask), FP);
  if constexpr (sizeof(Real) == 4) {
    const float4 xr = reinterpret_cast<const float4 *>(P.xr32)[sidx];
    const float x = xr.x + eoff_a(o) * (float)P.g.h[0];
    const float y = xr.y + eoff_b(o) * (float)P.g.h[1];
    const float z = (DIM == 3) ? xr.z + eoff_e(DIM, o) * (float)P.g.h[2] : 0.f;
    rec[0] = x; rec[1] = x; rec[2] = y; rec[3] = y; rec[4] = z; rec[5] = z; rec[6] = 0.f; rec[7] = 0.f;
  } else {
    rec[0] = P.xs64[(size_t)sidx * DIM + 0];
    rec[1] = P.xs64[(size_t)sidx * DIM + 1];
    rec[2] = (DIM == 3) ? P.xs64[(size_t)sidx * DIM + 2] : 0.0;
    rec[3] = 0.0;
  }
  /* coefficients field-major (field f, j-th involved patch), each repeated edup() times */
  constexpr int H = ehead<Real>(), D = edup<Real>();
  const int NI = epopc(mask);
  int j = 0;
  for (int k = 0; k < NEN; k++) {
    if (!((mask >> k) & 1)) continue;
    if (setup[k]) {
      const long long pos = P.coff[node[k]] + P.slot[node[k] * 8 + eslot(DIM, k, o)] + pp;
      const size_t src = (size_t)pos * P.F + P.f0;
      for (int f = 0; f < FP; f++) {
        Real c;
        if constexpr (sizeof(Real) == 4) c = P.c32[src + f];
        else c = P.c64[src + f];
        for (int q = 0; q < D; q++) rec[H + (f * NI + j) * D + q] = c;
      }
    } else {
      for (int f = 0; f < FP; f++)
        for (int q = 0; q < D; q++) rec[H + (f * NI + j) * D + q] = Real(0);
    }
    j++;
  }
  for (int q = H + NI * FP * D; q < S; q++) rec[q] = Real(0);
}

/* Per-CTA description of a cell's evaluation block: neighbour counts, first sorted index, corner
   nodes and their set-up state. */
template <int DIM>
__device__ __forceinline__ void cell_block(const EvalParams &P, int cell, int *s_cnt, int *s_first, int *s_node,
                                           int *s_setup)
{
  constexpr int NEN = EGeo<DIM>::NEN, NOFF = EGeo<DIM>::NOFF;
  const lgb_geom &g = P.g;
  const int tid = threadIdx.x;
  int ci, cj, cl;
  lgb_cell_ijk(g, cell, ci, cj, cl);
  if (tid < NOFF) {
    int ni = ci + eoff_a(tid), nj = cj + eoff_b(tid), nl = cl + eoff_e(DIM, tid);
    int cnt = 0, first = 0;
    if (ni >= 0 && ni < g.nc[0] && nj >= 0 && nj < g.nc[1] && nl >= 0 && nl < g.nc[2]) {
      int nb = ni + nj * g.nc[0] + nl * g.nc[0] * g.nc[1];
      first = P.cstart[nb];
      cnt = P.cstart[nb + 1] - first;
    }
    s_cnt[tid] = cnt;
    s_first[tid] = first;
  }
  if (tid < NEN) {
    int node = (ci + ecorner_ox(tid)) + (cj + ecorner_oy(tid)) * g.n[0] + (cl + ecorner_oz(DIM, tid)) * g.n[0] * g.n[1];
    s_node[tid] = node;
    s_setup[tid] = P.setup[node];
  }
}

/* Builds the staged record blocks of every cell into P.rec32 (FP32, FP fields from field f0), in
   neighbour-offset order, at P.rec_off[cell].  Runs only when `force` or when the preceding
   factorisation launch set up or solved at least one patch (device-side count), so the launch can
   sit in the captured step graph. */
template <int DIM, int FP>
__global__ void __launch_bounds__(128) k_build_records(EvalParams P, int force)
{
  constexpr int NOFF = EGeo<DIM>::NOFF;
  __shared__ int s_cnt[27], s_first[27], s_node[8], s_setup[8];
  if (!force && P.ctrl->nwork == 0) return;
  for (int cell = blockIdx.x; cell < P.g.ncells; cell += gridDim.x) {
    cell_block<DIM>(P, cell, s_cnt, s_first, s_node, s_setup);
    __syncthreads();
    float *dst = P.rec32 + P.rec_off[cell];
    for (int o = 0; o < NOFF; o++) {
      const int S = erec<float>(epopc(einv_mask(DIM, o)), FP);
      for (int p = threadIdx.x; p < s_cnt[o]; p += blockDim.x)
        write_record<float, DIM, FP>(P, o, p, s_first[o] + p, s_node, s_setup, dst + (size_t)p * S);
      dst += (size_t)s_cnt[o] * S;
    }
    __syncthreads();
  }
}

/* shared-memory address of a generic pointer (PTX operands) */
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

/* Round planner (one thread): packs the next records of the block, in neighbour order, into a
   staging buffer of `budget` elements; advances the cursor (o, pp) and returns the elements planned. */
template <typename Real, int DIM, int FP>
__device__ __noinline__ int eval_plan(const int *cnt, int budget, int &o, int &pp, int *seg_o, int *seg_p0, int *seg_n,
                                      int *seg_base, int *nseg_out)
{
  constexpr int NOFF = EGeo<DIM>::NOFF;
  int base = 0, nseg = 0;
  while (o < NOFF) {
    int c = cnt[o] - pp;
    if (c <= 0) { o++; pp = 0; continue; }
    int S = erec<Real>(epopc(einv_mask(DIM, o)), FP);
    int fit = (budget - base) / S;
    if (fit <= 0) break;
    int take = min(c, fit);
    seg_o[nseg] = o; seg_p0[nseg] = pp; seg_n[nseg] = take; seg_base[nseg] = base;
    nseg++;
    base += take * S;
    pp += take;
    if (pp >= cnt[o]) { o++; pp = 0; }
  }
  *nseg_out = nseg;
  return base;
}

/* The gather evaluation (FP64 path, and FP32 where no record blocks exist): each round the CTA
   gathers the next records of the block from the coefficient pool into shared memory (any
   precision, any field range), then every thread evaluates its particles against them. */
template <typename Real, int DIM, int FP, int R, int KER>
__global__ void __launch_bounds__(LGB_CHUNK_MAX / R) k_eval(EvalParams P)
{
  constexpr int NEN = EGeo<DIM>::NEN, NOFF = EGeo<DIM>::NOFF;
  const int EVAL_T = blockDim.x; /* work-unit capacity = EVAL_T * R particles (P.chunk_cap) */
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real *sm = reinterpret_cast<Real *>(smem_raw);
  __shared__ int s_cnt[27], s_first[27], s_node[8], s_setup[8];
  __shared__ int s_seg_o[1][27], s_seg_p0[1][27], s_seg_n[1][27], s_seg_base[1][27], s_nseg[1];
  __shared__ long long s_pre[28];
  __shared__ int s_o, s_pp, s_cell, s_pbeg, s_pn, s_blk, s_wsum;
  const lgb_geom &g = P.g;
  const int tid = threadIdx.x;
  const int chunk = blockIdx.x;
  const int total = P.chunk_start[g.ncells];
  if (chunk >= total) return;
  if (tid == 0) {
    int lo = 0, hi = g.ncells - 1;           /* last cell with chunk_start[c] <= chunk */
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (P.chunk_start[mid] <= chunk) lo = mid; else hi = mid - 1;
    }
    int c = lo;
    int q = chunk - P.chunk_start[c];
    int nch = P.chunk_start[c + 1] - P.chunk_start[c];
    int ncell = P.pstart[c + 1] - P.pstart[c];
    /* the cell's particles are split evenly over its work units (no nearly empty last unit) */
    int b0 = (int)(((long long)ncell * q) / nch), b1 = (int)(((long long)ncell * (q + 1)) / nch);
    s_cell = c;
    s_pbeg = P.pstart[c] + b0;
    s_pn = b1 - b0;
    s_wsum = 0;
    s_o = 0;
    s_pp = 0;
  }
  __syncthreads();
  const int cell = s_cell;
  int ci, cj, cl;
  lgb_cell_ijk(g, cell, ci, cj, cl);
  cell_block<DIM>(P, cell, s_cnt, s_first, s_node, s_setup);
  __syncthreads();
  if (tid == 0) {
    long long b = 0;
    for (int o = 0; o < NOFF; o++) {
      s_pre[o] = b;
      b += (long long)s_cnt[o] * erec<Real>(epopc(einv_mask(DIM, o)), FP);
    }
    s_pre[NOFF] = b;
    int nb = 0;
    for (int o = 0; o < NOFF; o++) nb += s_cnt[o];
    s_blk = nb;
  }
  __syncthreads();
  if (s_blk == 0) return; /* empty neighbourhood: the value is left untouched (interpolation.c:89) */

  /* particles of this work unit */
  const int pn = s_pn;
  int pid[R];
  Real px[R][3];
#pragma unroll
  for (int r = 0; r < R; r++) {
    int idx = tid * R + r; /* consecutive particles per thread: active threads fill whole warps */
    pid[r] = (idx < pn) ? P.plist[s_pbeg + idx] : -1;
    int cc[3] = {ci, cj, cl};
    for (int d = 0; d < 3; d++) {
      double xv = 0.0;
      if (d < DIM && pid[r] >= 0) xv = P.xp[(size_t)pid[r] * DIM + d];
      if constexpr (sizeof(Real) == 4) px[r][d] = (d < DIM) ? (float)(xv - (g.O[d] + g.h[d] * cc[d])) : 0.f;
      else px[r][d] = xv;
    }
  }
  /* warps without particles stage records and meet the barriers but skip the arithmetic */
  const bool warp_active = __any_sync(0xffffffffu, pid[0] >= 0);
  Real acc[R][NEN][FP];
#pragma unroll
  for (int r = 0; r < R; r++)
#pragma unroll
    for (int k = 0; k < NEN; k++)
#pragma unroll
      for (int f = 0; f < FP; f++) acc[r][k][f] = Real(0);

  /* shared memory: [staging buffer] [FP32 running sums: one block of R*NEN*FP (+1 pad, odd stride:
     no bank conflicts) floats per thread] */
  const int nbuf = 1;
  constexpr int RUNB = R * NEN * FP + 1;
  float *run = reinterpret_cast<float *>(sm + (size_t)nbuf * P.budget) + (size_t)tid * RUNB;
  const int rstride = 0;
  if constexpr (sizeof(Real) == 4) {
#pragma unroll
    for (int q = 0; q < R * NEN * FP; q++) run[q] = 0.f;
  }
  const Real eps = (Real)g.eps_r;
  const Real ga = (Real)(-(g.eps_r * g.eps_r) * 1.4426950408889634);
  const int kernel = g.kernel;

  for (;;) {
    if (tid == 0) {
      int o = s_o, pp = s_pp;
      eval_plan<Real, DIM, FP>(s_cnt, P.budget, o, pp, s_seg_o[0], s_seg_p0[0], s_seg_n[0], s_seg_base[0], &s_nseg[0]);
      s_o = o; s_pp = pp;
    }
    __syncthreads();
    const int nseg = s_nseg[0];
    if (nseg == 0) break;
    for (int sgi = 0; sgi < nseg; sgi++) {
      const int o = s_seg_o[0][sgi], p0 = s_seg_p0[0][sgi], n = s_seg_n[0][sgi];
      const int S = erec<Real>(epopc(einv_mask(DIM, o)), FP);
      Real *rbase = sm + s_seg_base[0][sgi];
      for (int p = tid; p < n; p += EVAL_T)
        write_record<Real, DIM, FP>(P, o, p0 + p, s_first[o] + p0 + p, s_node, s_setup, rbase + (size_t)p * S);
    }
    __syncthreads();
    if (warp_active)
      for (int sgi = 0; sgi < nseg; sgi++)
        eval_dispatch<Real, DIM, FP, R, KER>(s_seg_o[0][sgi], sm + s_seg_base[0][sgi], s_seg_n[0][sgi], px, acc,
                                              eps, ga, kernel, run, rstride);
    __syncthreads();
  }

  /* epilogue: PU weights and the weighted sum */
  int wloc = 0;
#pragma unroll
  for (int r = 0; r < R; r++) {
    if (pid[r] < 0) continue;
    Real pw[NEN];
    double den;
    int ns;
    double xabs[3];
    for (int d = 0; d < 3; d++) xabs[d] = (d < DIM) ? P.xp[(size_t)pid[r] * DIM + d] : 0.0;
    eval_weights<Real, DIM>(g, ci, cj, cl, xabs, px[r], pw, den, ns);
    wloc += ns;
    double *o = P.out + (size_t)pid[r] * P.out_stride;
    if constexpr (sizeof(Real) == 4) {
      double inv = (den > 0.0) ? 1.0 / den : 0.0;
#pragma unroll
      for (int f = 0; f < FP; f++) {
        float hi = 0.f, lo = 0.f;
#pragma unroll
        for (int k = 0; k < NEN; k++) {
          const float Ik = run[(r * NEN + k) * FP + f];
          float prod = pw[k] * Ik;
          float perr = fmaf(pw[k], Ik, -prod);
          lgb_df_add(hi, lo, prod);
          lo += perr;
        }
        o[f] = ((double)hi + (double)lo) * inv;
      }
    } else {
      double val[FP];
#pragma unroll
      for (int f = 0; f < FP; f++) val[f] = 0.0;
#pragma unroll
      for (int k = 0; k < NEN; k++) {
        double w = (den > 0.0) ? (double)pw[k] / den : 0.0;
#pragma unroll
        for (int f = 0; f < FP; f++) val[f] += (double)acc[r][k][f] * w;
      }
#pragma unroll
      for (int f = 0; f < FP; f++) o[f] = val[f];
    }
  }
  /* algorithmic work of this unit: distances 10 flops, kernel k_phi, 2 flops per coefficient FMA,
     18 per support node of the weights, 2F+1 per corner in the epilogue */
  for (int off = 16; off > 0; off >>= 1) wloc += __shfl_down_sync(0xffffffffu, wloc, off);
  if ((tid & 31) == 0) atomicAdd(&s_wsum, wloc);
  __syncthreads();
  if (tid == 0) {
    long long msum = 0;
    for (int o = 0; o < NOFF; o++) {
      int mask = einv_mask(DIM, o), ninv = 0;
      for (int k = 0; k < NEN; k++) ninv += ((mask >> k) & 1) && s_setup[k];
      msum += (long long)s_cnt[o] * ninv;
    }
    double kphi = (KER == KER_GAUSS || g.kernel == LGB_KERNEL_GAUSSIAN) ? 4.0 : 8.0;
    double fl = (double)pn * ((double)s_blk * (10.0 + kphi) + 2.0 * FP * (double)msum + NEN * (2.0 * FP + 1.0)) +
                18.0 * (double)s_wsum;
    double by = (double)pn * (8.0 * DIM + 4.0 + 8.0 * FP) +
                (double)s_blk * (sizeof(Real) == 4 ? 16.0 : 8.0 * DIM) + (double)msum * FP * sizeof(Real);
    atomicAdd(&P.ctrl->eval_flops, fl);
    atomicAdd(&P.ctrl->eval_bytes, by);
  }
}

/* FP64 PU weights of every live particle (output of the "weights" field). */
template <int DIM>
__global__ void k_weights(lgb_geom g, int np, const double *__restrict__ xp, const int *__restrict__ cell,
                          const int *__restrict__ alive, double *__restrict__ w)
{
  constexpr int NEN = EGeo<DIM>::NEN;
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np || !alive[p] || cell[p] < 0) return;
  int ci, cj, cl;
  lgb_cell_ijk(g, cell[p], ci, cj, cl);
  double x[3] = {xp[(size_t)p * DIM], xp[(size_t)p * DIM + 1], DIM == 3 ? xp[(size_t)p * DIM + 2] : 0.0};
  double pw[NEN], den;
  int ns;
  eval_weights<double, DIM>(g, ci, cj, cl, x, x, pw, den, ns);
  for (int k = 0; k < NEN; k++) w[(size_t)p * NEN + k] = (den > 0.0) ? pw[k] / den : 0.0;
}
