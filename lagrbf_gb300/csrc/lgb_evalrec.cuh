/*
 * lgb_evalrec.cuh -- FP32 PU evaluation from precomputed record blocks: the hot kernel of the
 * FP32-evaluation path (RBFInterpolation -> PointwiseInterpolation_AVX512,
 * src/interpolation/interpolation_avx512.c:121-291, with the PU weights of
 * SwarmInterpSetWeights, src/swarm/weights_avx.c:97-243).
 *
 * Record blocks.  For every cell, the data points of its 3^dim neighbour cells are stored once as a
 * contiguous stream of records, in the reference's neighbour order, points of a cell in cell
 * order.  In 3D the centre cell (in all eight corner patches) appears twice, as two "virtual
 * segments" carrying the coefficients of corners 0-3 and of corners 4-7, so that no record holds
 * more than four patches; 2D has no split.  A record is
 *     { x', x', y', y', [z', z'], (X_k[j, f], X_k[j, f]) for field f, involved corner k ... }
 * with x' = eps_r * (x - origin of the evaluating cell) rounded from FP64 (Gaussian kernel: unscaled,
 * whose FP32 error measured lower that way), every value twice so that one 64-bit register pair
 * holds it for the two particles a thread evaluates, padded to 16 bytes.
 *
 * Arithmetic per (particle pair, data point), all on packed FP32 pairs (PTX f32x2):
 *     d2 = |p' - x'|^2 + 1e-30                   (eps_r folded into the coordinates)
 *     w  = min(d2 * rsqrt(d2) - 1, 0)            (= eps_r r - 1; rsqrt.approx, one MUFU op per lane)
 *     phi = w^4 (4 w + 5)                        (Wendland C2: (1 - eps r)^4 (4 eps r + 1))
 *     acc[f][k] += phi * X_k[j, f]
 * The 1e-30 keeps rsqrt finite at d2 = 0 and is below the rounding of every other d2.  The PU
 * weights w_k (Wendland C2 of the corner distances over the support sum, normalised in FP64) are
 * computed before the loop; at the end of each segment (the points of one neighbour cell) its
 * per-patch sums are folded into the particle's field sums as sum_k w_k acc[f][k] with an
 * error-free TwoSum (blocked, compensated accumulation of v = sum_k w_k sum_j phi_j X_k[j], the
 * inner sums split by neighbour cell).  Per thread this keeps 2 x F compensated sums in registers
 * instead of 2 x 2^dim x F per-patch sums.
 *
 * Staging.  A ring of four shared-memory stages is filled by cp.async.bulk with mbarrier completion.
 * Warps consume stages independently: after a stage each warp adds one to the stage's release
 * count, and the warp that releases it last plans the next round of records into it and issues the
 * copy, so no block-wide barrier separates rounds.  Every wait is bounded; a wait that gives up sets
 * the context's eval_error, its warp leaves the loop, and before the block exits thread 0 waits
 * (bounded) for the copies still in flight into its shared memory.
 */
#pragma once
#include "lgb_eval.cuh"

__host__ __device__ constexpr int vs_off(int dim, int vs) { return (dim == 3 && vs > 13) ? vs - 1 : vs; }
__host__ __device__ constexpr int vs_mask(int dim, int vs)
{
  return einv_mask(dim, vs_off(dim, vs)) & ((dim == 3 && vs == 13) ? 0x0F : (dim == 3 && vs == 14) ? 0xF0 : 0xFF);
}
template <int DIM> struct VGeo { static constexpr int NVS = LGB_NVSEG(DIM); };
/* Coordinate scale of the records and particles: eps_r (folded into the distance), except for the
   Gaussian kernel, evaluated as 2^(-eps_r^2 log2(e) d2) on unscaled coordinates. */
__host__ __device__ __forceinline__ double evr_scale(const lgb_geom &g)
{
  return g.kernel == LGB_KERNEL_GAUSSIAN ? 1.0 : g.eps_r;
}

#include "lgb_eval_tune.h"
#ifndef EVR_NB
#define EVR_NB LGB_EVR_NB_TUNED /* stages in the ring (measured table) */
#endif
#ifndef LGB_EVR_UNROLL
#define LGB_EVR_UNROLL 4 /* points of a segment in flight per thread */
#endif

/* Bounded wait for the phase `parity` of an mbarrier (every polling thread acquires the completed
   copy); false if it did not complete within `limit` polls. */
__device__ __forceinline__ bool evr_wait(unsigned long long *mbar, unsigned parity, int limit)
{
  const unsigned mb = smem_addr(mbar);
  for (int it = 0; it < limit; ++it) {
    unsigned done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(mb), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

struct EvrShared {
  unsigned long long full[EVR_NB];
  int rel[EVR_NB], nseg[EVR_NB], phases[EVR_NB];
  int seg_vs[EVR_NB][28], seg_n[EVR_NB][28], seg_base[EVR_NB][28], seg_flags[EVR_NB][28];
  int cnt[27], first[27], node[8], setup[8];
  int vcnt[28], vlen[28];
  long long vpre[29];
  long long src0;      /* stream start of the cell (floats) */
  int vs, pp;          /* planner cursor */
  int abort_, cell, pbeg, pn, blk, wsum;
};

/* Plans the next round of records of the stream into stage b and arms the stage: a bulk copy with
   its byte count, or a plain arrival when the stream is exhausted (the stage then reads nseg 0).
   Called by one thread; rounds are planned in order (see the release protocol above).  Each planned
   piece of a virtual segment carries flags: 1 = its first records, 2 = its last. */
template <int DIM>
__device__ __noinline__ void evr_plan_issue(const EvalParams &P, EvrShared &S, float *ring, int b)
{
  constexpr int NVS = VGeo<DIM>::NVS;
  int vs = S.vs, pp = S.pp;
  while (vs < NVS && pp >= S.vcnt[vs]) { vs++; pp = 0; }
  const long long pos = (vs < NVS) ? S.vpre[vs] + (long long)pp * S.vlen[vs] : 0;
  int base = 0, nseg = 0;
  while (vs < NVS) {
    const int c = S.vcnt[vs] - pp;
    if (c <= 0) { vs++; pp = 0; continue; }
    const int len = S.vlen[vs];
    const int fit = (P.budget - base) / len;
    if (fit <= 0) break;
    const int take = c < fit ? c : fit;
    S.seg_vs[b][nseg] = vs;
    S.seg_n[b][nseg] = take;
    S.seg_base[b][nseg] = base;
    S.seg_flags[b][nseg] = (pp == 0 ? 1 : 0) | (pp + take >= S.vcnt[vs] ? 2 : 0);
    nseg++;
    base += take * len;
    pp += take;
    if (pp >= S.vcnt[vs]) { vs++; pp = 0; }
  }
  S.vs = vs;
  S.pp = pp;
  S.nseg[b] = nseg;
  S.phases[b]++;
  const unsigned mb = smem_addr(&S.full[b]);
  if (base > 0) {
    const unsigned bytes = (unsigned)base * 4u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
    if (!P.withhold_copies) {
      const float *src = P.rec32 + S.src0 + pos;
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   ::"r"(smem_addr(ring + (size_t)b * P.budget)), "l"(src), "r"(bytes), "r"(mb) : "memory");
    }
  } else {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mb) : "memory");
  }
}

/* n records of NI patches at rec (shared memory), both particles of the thread, added to the first
   NI columns of acc. */
template <int DIM, int FP, int KER, int NI>
__device__ __forceinline__ void evr_body(const float *__restrict__ rec, int n, f32x2 pxx, f32x2 pyy, f32x2 pzz,
                                         f32x2 (&acc)[FP][4], int kernel, float ga)
{
  constexpr int S = LGB_REC2_LEN(DIM, NI, FP);
  constexpr int H = 2 * DIM;
  constexpr int NV = S / 4;
  const f32x2 tiny = x2_pack(1e-30f, 1e-30f), mone = x2_pack(-1.f, -1.f);
  const f32x2 four = x2_pack(4.f, 4.f), five = x2_pack(5.f, 5.f);
  LGB_UNROLL(LGB_EVR_UNROLL)
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
      d2 = x2_fma(dx, dx, x2_fma(dy, dy, x2_fma(dz, dz, tiny)));
    } else {
      d2 = x2_fma(dx, dx, x2_fma(dy, dy, tiny));
    }
    float d2a, d2b;
    x2_unpack(d2, d2a, d2b);
    f32x2 ph;
    if constexpr (KER == KER_C2) {
      float ra, rb;
      asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(ra) : "f"(d2a));
      asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(d2b));
      float wa, wb;
      x2_unpack(x2_fma(d2, x2_pack(ra, rb), mone), wa, wb); /* eps r - 1 */
      const f32x2 w = x2_pack(fminf(wa, 0.f), fminf(wb, 0.f));
      const f32x2 w2 = x2_mul(w, w);
      ph = x2_mul(x2_mul(w2, w2), x2_fma(w, four, five));
    } else if constexpr (KER == KER_GAUSS) {
      ph = x2_pack(exp2f(ga * d2a), exp2f(ga * d2b)); /* ga = -eps_r^2 log2(e) */
    } else {
      ph = x2_pack(lgb_phi<float>(kernel, sqrtf(d2a), 1.f), lgb_phi<float>(kernel, sqrtf(d2b), 1.f));
    }
#pragma unroll
    for (int f = 0; f < FP; f++)
#pragma unroll
      for (int j = 0; j < NI; j++)
        acc[f][j] = x2_fma(ph, x2_pack(v[H + 2 * (f * NI + j)], v[H + 2 * (f * NI + j) + 1]), acc[f][j]);
  }
}

/* Folds a segment's per-patch sums into the particle pair's PU-weighted field sums:
   (hi, lo)[f] += w_k * acc[f][j] for every involved corner k (W: this thread's weights, one pair per
   corner), accumulated with an error-free TwoSum so that the field sum carries no rounding error
   beyond that of the per-segment sums and of the products. */
template <int FP, int NI>
__device__ __forceinline__ void evr_flush(const f32x2 *W, int mask, const f32x2 (&acc)[FP][4], f32x2 (&hi)[FP],
                                          f32x2 (&lo)[FP])
{
  unsigned m = (unsigned)mask;
#pragma unroll
  for (int j = 0; j < NI; j++) {
    const int k = __ffs(m) - 1;
    m &= m - 1;
    const f32x2 w = W[k];
#pragma unroll
    for (int f = 0; f < FP; f++) {
      const f32x2 p = x2_mul(w, acc[f][j]);
      const f32x2 s = x2_add(hi[f], p);
      const f32x2 bb = x2_sub(s, hi[f]);
      const f32x2 e = x2_add(x2_sub(hi[f], x2_sub(s, bb)), x2_sub(p, bb));
      lo[f] = x2_add(lo[f], e);
      hi[f] = s;
    }
  }
}

/* One planned piece of virtual segment vs: n records at rec.  A segment split over several stages
   keeps its sums in acc between pieces; they start at zero with its first piece (flags & 1) and
   are folded in with its last (flags & 2), so every segment is one block of the accumulation. */
template <int DIM, int FP, int KER>
__device__ __forceinline__ void evr_piece(int vs, int flags, const float *rec, int n, f32x2 pxx, f32x2 pyy,
                                          f32x2 pzz, const f32x2 *W, f32x2 (&acc)[FP][4], f32x2 (&hi)[FP],
                                          f32x2 (&lo)[FP], int kernel, float ga)
{
  const int mask = vs_mask(DIM, vs);
  if (flags & 1) {
#pragma unroll
    for (int f = 0; f < FP; f++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[f][j] = 0ull;
  }
  switch (__popc(mask)) {
  case 1:
    evr_body<DIM, FP, KER, 1>(rec, n, pxx, pyy, pzz, acc, kernel, ga);
    if (flags & 2) evr_flush<FP, 1>(W, mask, acc, hi, lo);
    break;
  case 2:
    evr_body<DIM, FP, KER, 2>(rec, n, pxx, pyy, pzz, acc, kernel, ga);
    if (flags & 2) evr_flush<FP, 2>(W, mask, acc, hi, lo);
    break;
  case 4:
    evr_body<DIM, FP, KER, 4>(rec, n, pxx, pyy, pzz, acc, kernel, ga);
    if (flags & 2) evr_flush<FP, 4>(W, mask, acc, hi, lo);
    break;
  default: break;
  }
}

/* Builds the record blocks into P.rec32 at P.rec_off[cell] (FP fields from field 0): every cell when
   `force`, else the cells marked in P.cdirty (the cells around the patches the preceding set-up /
   solve launch processed: their records carry those patches' coefficients), and only when that
   launch processed at least one patch (device-side count), so the launch can sit in the captured
   step graph.  Marks are cleared as the cells are rebuilt. */
template <int DIM, int FP>
__global__ void __launch_bounds__(128) k_build_records2(EvalParams P, int force)
{
  constexpr int NVS = VGeo<DIM>::NVS, NEN = EGeo<DIM>::NEN;
  __shared__ int s_cnt[27], s_first[27], s_node[8], s_setup[8];
  if (!force && P.ctrl->nwork == 0) return;
  const lgb_geom &g = P.g;
  const double eps = evr_scale(g);
  for (int cell = blockIdx.x; cell < g.ncells; cell += gridDim.x) {
    if (!force && !P.cdirty[cell]) continue; /* the same for the whole block */
    cell_block<DIM>(P, cell, s_cnt, s_first, s_node, s_setup);
    __syncthreads();
    int ci, cj, cl;
    lgb_cell_ijk(g, cell, ci, cj, cl);
    const double org[3] = {g.O[0] + g.h[0] * ci, g.O[1] + g.h[1] * cj, DIM == 3 ? g.O[2] + g.h[2] * cl : 0.0};
    float *dst = P.rec32 + P.rec_off[cell];
    for (int vs = 0; vs < NVS; vs++) {
      const int o = vs_off(DIM, vs), mask = vs_mask(DIM, vs), ni = __popc(mask);
      const int S = LGB_REC2_LEN(DIM, ni, FP);
      for (int p = threadIdx.x; p < s_cnt[o]; p += blockDim.x) {
        const int sidx = s_first[o] + p;
        float *rec = dst + (size_t)p * S;
        for (int d = 0; d < DIM; d++) {
          const float x = (float)(eps * (P.xs64[(size_t)sidx * DIM + d] - org[d]));
          rec[2 * d] = x;
          rec[2 * d + 1] = x;
        }
        for (int f = 0; f < FP; f++) {
          int j = 0;
          for (int k = 0; k < NEN; k++) {
            if (!((mask >> k) & 1)) continue;
            float c = 0.f;
            if (s_setup[k]) {
              const long long pos = P.coff[s_node[k]] + P.slot[s_node[k] * 8 + eslot(DIM, k, o)] + p;
              c = P.c32[(size_t)pos * P.F + f];
            }
            rec[2 * DIM + 2 * (f * ni + j)] = c;
            rec[2 * DIM + 2 * (f * ni + j) + 1] = c;
            j++;
          }
        }
        for (int q = 2 * DIM + 2 * ni * FP; q < S; q++) rec[q] = 0.f;
      }
      dst += (size_t)s_cnt[o] * S;
    }
    __syncthreads();
    if (threadIdx.x == 0) P.cdirty[cell] = 0;
  }
}

/* The FP32 evaluation of FP (= dim) fields from the record blocks.  One CTA per work unit (up to
   2 * blockDim.x particles of one cell, two per thread). */
template <int DIM, int FP, int KER>
__global__ void __launch_bounds__(LGB_CHUNK_MAX / 2) k_eval_rec(EvalParams P)
{
  constexpr int NEN = EGeo<DIM>::NEN, NOFF = EGeo<DIM>::NOFF, NVS = VGeo<DIM>::NVS, NB = EVR_NB;
  constexpr int WS = NEN + 1; /* weight pairs per thread; odd stride: conflict-free 8-byte accesses */
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ EvrShared S;
  float *ring = reinterpret_cast<float *>(smem_raw);
  const lgb_geom &g = P.g;
  const int tid = threadIdx.x, lane = tid & 31, nwarps = blockDim.x >> 5;
  const int chunk = blockIdx.x;
  const int total = P.chunk_start[g.ncells];
  if (chunk >= total) return;
  if (tid < 32) {
    /* the work unit's cell: the last cell c with chunk_start[c] <= chunk (a 32-way search) */
    int lo = 0, hi = g.ncells - 1;
    while (hi > lo) {
      const int step = (hi - lo + 32) / 32;
      const int c = min(lo + lane * step, hi);
      const unsigned le = __ballot_sync(0xffffffffu, P.chunk_start[c] <= chunk);
      const int last = 31 - __clz(le); /* chunk_start is non-decreasing and chunk_start[lo] <= chunk */
      const int nlo = min(lo + last * step, hi);
      hi = min(nlo + step - 1, hi);
      lo = nlo;
      if (step == 1) hi = lo;
    }
    if (tid == 0) {
      const int c = lo;
      const int q = chunk - P.chunk_start[c];
      const int nch = P.chunk_start[c + 1] - P.chunk_start[c];
      const int ncell = P.pstart[c + 1] - P.pstart[c];
      const int b0 = (int)(((long long)ncell * q) / nch), b1 = (int)(((long long)ncell * (q + 1)) / nch);
      S.cell = c;
      S.pbeg = P.pstart[c] + b0;
      S.pn = b1 - b0;
      S.wsum = 0;
      S.abort_ = 0;
      S.vs = 0;
      S.pp = 0;
      S.src0 = P.rec_off[c];
    }
  }
  __syncthreads();
  const int cell = S.cell;
  int ci, cj, cl;
  lgb_cell_ijk(g, cell, ci, cj, cl);
  cell_block<DIM>(P, cell, S.cnt, S.first, S.node, S.setup);
  __syncthreads();
  if (tid < NVS) {
    S.vcnt[tid] = S.cnt[vs_off(DIM, tid)];
    S.vlen[tid] = LGB_REC2_LEN(DIM, __popc(vs_mask(DIM, tid)), FP);
  }
  __syncthreads();
  if (tid == 0) {
    long long b = 0;
    int nb = 0;
    for (int vs = 0; vs < NVS; vs++) {
      S.vpre[vs] = b;
      b += (long long)S.vcnt[vs] * S.vlen[vs];
    }
    S.vpre[NVS] = b;
    for (int o = 0; o < NOFF; o++) nb += S.cnt[o];
    S.blk = nb;
    if (nb > 0) {
      for (int i = 0; i < NB; i++) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&S.full[i])) : "memory");
        S.rel[i] = 0;
        S.phases[i] = 0;
      }
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      for (int i = 0; i < NB; i++) evr_plan_issue<DIM>(P, S, ring, i);
    }
  }
  __syncthreads();
  if (S.blk == 0) return; /* empty neighbourhood: the value is left untouched (interpolation.c:89) */

  /* the thread's two particles (consecutive in the unit), coordinates relative to the cell origin */
  const int pn = S.pn;
  int pid[2];
  float pxs[2][3], pxr[2][3]; /* scaled (as the records) and plain relative coordinates */
  const int cc[3] = {ci, cj, cl};
#pragma unroll
  for (int r = 0; r < 2; r++) {
    const int idx = 2 * tid + r;
    pid[r] = (idx < pn) ? P.plist[S.pbeg + idx] : -1;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double rel = 0.0;
      if (d < DIM && pid[r] >= 0) rel = P.xp[(size_t)pid[r] * DIM + d] - (g.O[d] + g.h[d] * cc[d]);
      pxs[r][d] = (float)(evr_scale(g) * rel);
      pxr[r][d] = (float)rel;
    }
  }
  const bool warp_active = __any_sync(0xffffffffu, pid[0] >= 0);
  const f32x2 pxx = x2_pack(pxs[0][0], pxs[1][0]), pyy = x2_pack(pxs[0][1], pxs[1][1]);
  const f32x2 pzz = x2_pack(pxs[0][2], pxs[1][2]);
  /* PU weights first (w_k = phiW_k / sum over the support, normalised in FP64), kept as pairs in
     this thread's shared-memory block: segments fold their patch sums in with them */
  f32x2 *W = reinterpret_cast<f32x2 *>(ring + (size_t)NB * P.budget) + (size_t)tid * WS;
  int wloc = 0;
  {
    float w[2][NEN];
#pragma unroll
    for (int r = 0; r < 2; r++) {
#pragma unroll
      for (int k = 0; k < NEN; k++) w[r][k] = 0.f;
      if (pid[r] < 0) continue;
      float pw[NEN];
      double den, xabs[3];
      int ns;
      for (int d = 0; d < 3; d++) xabs[d] = (d < DIM) ? P.xp[(size_t)pid[r] * DIM + d] : 0.0;
      eval_weights<float, DIM>(g, ci, cj, cl, xabs, pxr[r], pw, den, ns);
      wloc += ns;
      const double inv = (den > 0.0) ? 1.0 / den : 0.0;
#pragma unroll
      for (int k = 0; k < NEN; k++) w[r][k] = (float)((double)pw[k] * inv);
    }
#pragma unroll
    for (int k = 0; k < NEN; k++) W[k] = x2_pack(w[0][k], w[1][k]);
  }
  f32x2 hi[FP], lo[FP], acc[FP][4];
#pragma unroll
  for (int f = 0; f < FP; f++) { hi[f] = 0ull; lo[f] = 0ull; }
  const int kernel = g.kernel;
  const float ga = (float)(-(g.eps_r * g.eps_r) * 1.4426950408889634);

  bool ok = true;
  for (int r = 0;; r++) {
    const int b = r % NB;
    if (!evr_wait(&S.full[b], (unsigned)((r / NB) & 1), P.poll_limit)) { ok = false; break; }
    const int nseg = S.nseg[b];
    if (nseg == 0) break;
    if (warp_active) {
      const float *buf = ring + (size_t)b * P.budget;
      for (int i = 0; i < nseg; i++)
        evr_piece<DIM, FP, KER>(S.seg_vs[b][i], S.seg_flags[b][i], buf + S.seg_base[b][i], S.seg_n[b][i], pxx, pyy,
                                pzz, W, acc, hi, lo, kernel, ga);
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      if (atomicAdd(&S.rel[b], 1) == nwarps - 1) { /* this warp releases the stage last: refill it */
        S.rel[b] = 0;
        __threadfence_block();
        evr_plan_issue<DIM>(P, S, ring, b);
      }
    }
  }
  if (!ok) {
    S.abort_ = 1;
    if (lane == 0) atomicExch(&P.ctrl->eval_error, 1);
  }
  __syncthreads();
  if (S.abort_) {
    /* copies may still be in flight into this block's stages: wait for them (bounded) before exit */
    if (tid == 0)
      for (int i = 0; i < NB; i++)
        if (S.phases[i] > 0) evr_wait(&S.full[i], (unsigned)((S.phases[i] - 1) & 1), P.poll_limit);
    return;
  }

  /* the PU-weighted field sums of the two particles */
#pragma unroll
  for (int r = 0; r < 2; r++) {
    if (pid[r] < 0) continue;
    double *o = P.out + (size_t)pid[r] * P.out_stride;
#pragma unroll
    for (int f = 0; f < FP; f++) {
      float h0, h1, l0, l1;
      x2_unpack(hi[f], h0, h1);
      x2_unpack(lo[f], l0, l1);
      o[f] = r ? (double)h1 + (double)l1 : (double)h0 + (double)l0;
    }
  }
  /* algorithmic work of this unit (the same count as the gather kernel) */
  for (int off = 16; off > 0; off >>= 1) wloc += __shfl_down_sync(0xffffffffu, wloc, off);
  if (lane == 0) atomicAdd(&S.wsum, wloc);
  __syncthreads();
  if (tid == 0) {
    long long msum = 0;
    for (int o = 0; o < NOFF; o++) {
      const int mask = einv_mask(DIM, o);
      int ninv = 0;
      for (int k = 0; k < NEN; k++) ninv += ((mask >> k) & 1) && S.setup[k];
      msum += (long long)S.cnt[o] * ninv;
    }
    const double kphi = (KER == KER_GAUSS || g.kernel == LGB_KERNEL_GAUSSIAN) ? 4.0 : 8.0;
    const double fl = (double)pn * ((double)S.blk * (10.0 + kphi) + 2.0 * FP * (double)msum + NEN * (2.0 * FP + 1.0)) +
                      18.0 * (double)S.wsum;
    const double by = (double)pn * (8.0 * DIM + 4.0 + 8.0 * FP) + (double)S.blk * 16.0 + (double)msum * FP * 4.0;
    atomicAdd(&P.ctrl->eval_flops, fl);
    atomicAdd(&P.ctrl->eval_bytes, by);
  }
}
