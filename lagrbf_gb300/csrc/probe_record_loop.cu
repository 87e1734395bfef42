/*
 * probe_record_loop.cu -- compute-only bound of the FP32 record loop of k_eval_rec (not part of the
 * library; built and run by lagrbf_gb300/probe_eval.py).
 *
 * The loop body of lgb_evalrec.cuh (packed FP32 pairs: distance, rsqrt, Wendland C2 polynomial,
 * per-patch FMAs for three fields and NI = 1, 2, 4 involved patches) runs over a block of records
 * held in shared memory for the whole kernel: no staging, no prologue or epilogue, no segment
 * bookkeeping.  RP particle pairs per thread (1: the library's layout; 2: the alternative with
 * twice the FMAs per shared load), U records unrolled.  Throughput is reported in particle-points
 * per second and as algorithmic TFLOP/s (18 + 6 NI flops per particle-point, the library's count)
 * against the FFMA peak given on the command line.
 */
#include <cstdio>
#include <cstdlib>
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 x2_pack(float a, float b) { f32x2 r; asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b)); return r; }
__device__ __forceinline__ void x2_unpack(f32x2 v, float &a, float &b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
__device__ __forceinline__ f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c) { f32x2 d; asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c)); return d; }
__device__ __forceinline__ f32x2 x2_mul(f32x2 a, f32x2 b) { f32x2 d; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
__device__ __forceinline__ f32x2 x2_sub(f32x2 a, f32x2 b) { f32x2 d; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }

template <int NI> struct L { static constexpr int S = ((6 + 2 * NI * 3) + 3) / 4 * 4; };

template <int RP, int NI, int U>
__global__ void kmb(const float *__restrict__ g, float *out, int n, int iters)
{
  constexpr int S = L<NI>::S, NV = S / 4;
  extern __shared__ __align__(16) float rec[];
  for (int i = threadIdx.x; i < n * S; i += blockDim.x) rec[i] = g[i];
  __syncthreads();
  f32x2 px[RP], py[RP], pz[RP], acc[RP][3][NI];
#pragma unroll
  for (int q = 0; q < RP; q++) {
    const float b = 0.01f * (threadIdx.x + 7 * q);
    px[q] = x2_pack(b, b + 0.1f); py[q] = x2_pack(b + 0.2f, b + 0.3f); pz[q] = x2_pack(b + 0.4f, b + 0.5f);
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
      for (int j = 0; j < NI; j++) acc[q][f][j] = 0ull;
  }
  const f32x2 tiny = x2_pack(1e-30f, 1e-30f), mone = x2_pack(-1.f, -1.f), four = x2_pack(4.f, 4.f), five = x2_pack(5.f, 5.f);
  for (int it = 0; it < iters; it++) {
#pragma unroll U
    for (int p = 0; p < n; ++p) {
      float v[S];
      const float4 *rv = reinterpret_cast<const float4 *>(rec + (size_t)p * S);
#pragma unroll
      for (int k = 0; k < NV; k++) { const float4 t = rv[k]; v[4*k] = t.x; v[4*k+1] = t.y; v[4*k+2] = t.z; v[4*k+3] = t.w; }
#pragma unroll
      for (int q = 0; q < RP; q++) {
        const f32x2 dx = x2_sub(px[q], x2_pack(v[0], v[1]));
        const f32x2 dy = x2_sub(py[q], x2_pack(v[2], v[3]));
        const f32x2 dz = x2_sub(pz[q], x2_pack(v[4], v[5]));
        const f32x2 d2 = x2_fma(dx, dx, x2_fma(dy, dy, x2_fma(dz, dz, tiny)));
        float a, b, ra, rb, wa, wb;
        x2_unpack(d2, a, b);
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(ra) : "f"(a));
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(b));
        x2_unpack(x2_fma(d2, x2_pack(ra, rb), mone), wa, wb);
        const f32x2 w = x2_pack(fminf(wa, 0.f), fminf(wb, 0.f));
        const f32x2 w2 = x2_mul(w, w);
        const f32x2 ph = x2_mul(x2_mul(w2, w2), x2_fma(w, four, five));
#pragma unroll
        for (int f = 0; f < 3; f++)
#pragma unroll
          for (int j = 0; j < NI; j++) acc[q][f][j] = x2_fma(ph, x2_pack(v[6 + 2 * (f * NI + j)], v[7 + 2 * (f * NI + j)]), acc[q][f][j]);
      }
    }
  }
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < RP; q++)
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
      for (int j = 0; j < NI; j++) { float a, b; x2_unpack(acc[q][f][j], a, b); s += a + b; }
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int RP, int NI, int U>
void run(int threads, const float *g, float *out, int nsm, double peak)
{
  constexpr int S = L<NI>::S;
  const int n = 2048 / S, iters = 400;
  const size_t smem = (size_t)n * S * 4 + 16384; /* + the rest of the real kernel's shared memory */
  cudaFuncSetAttribute(kmb<RP, NI, U>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kmb<RP, NI, U>, threads, smem);
  const int grid = nsm * per * 4;
  cudaFuncAttributes fa; cudaFuncGetAttributes(&fa, kmb<RP, NI, U>);
  kmb<RP, NI, U><<<grid, threads, smem>>>(g, out, n, 2);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  cudaEventRecord(e0);
  kmb<RP, NI, U><<<grid, threads, smem>>>(g, out, n, iters);
  cudaEventRecord(e1); cudaEventSynchronize(e1);
  float ms; cudaEventElapsedTime(&ms, e0, e1);
  const double pp = (double)grid * threads * RP * 2 * n * iters; /* particle-points */
  const double fl = pp * (18.0 + 6.0 * NI);
  printf("RP=%d NI=%d U=%d threads=%3d regs=%3d ctas/SM=%2d warps/SM=%2d: %.2f ms, %.2f Gpp/s, %.1f TFLOP/s = %.3f of peak\n",
         RP, NI, U, threads, fa.numRegs, per, per * threads / 32, ms, pp / ms / 1e6, fl / ms / 1e9, fl / ms / 1e9 / peak);
}

int main(int argc, char **argv)
{
  const double peak = argc > 1 ? atof(argv[1]) : 78.4;
  int dev = 0, nsm = 0; cudaGetDevice(&dev); cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  float *g, *out; cudaMalloc(&g, 4 * 4096); cudaMalloc(&out, 4 << 24);
  float h[4096]; for (int i = 0; i < 4096; i++) h[i] = 0.05f + 0.9f * ((i * 2654435761u) % 1000) / 1000.f;
  cudaMemcpy(g, h, sizeof h, cudaMemcpyHostToDevice);
  run<1, 1, 4>(96, g, out, nsm, peak); run<1, 2, 4>(96, g, out, nsm, peak); run<1, 4, 4>(96, g, out, nsm, peak);
  run<2, 1, 2>(64, g, out, nsm, peak); run<2, 2, 2>(64, g, out, nsm, peak); run<2, 4, 2>(64, g, out, nsm, peak);
  run<2, 1, 2>(32, g, out, nsm, peak); run<2, 2, 2>(32, g, out, nsm, peak); run<2, 4, 2>(32, g, out, nsm, peak);
  run<2, 4, 4>(64, g, out, nsm, peak); run<2, 4, 1>(64, g, out, nsm, peak);
  printf("%s\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
