// latency.cu -- microbenchmark of the operations on the SSA critical path
// on GB300: FP64 add/FMA/divide throughput and dependent-chain latency, the
// integer-pipe replacements used by the solver (si_div, si_log,
// si_neglog_u32, integer comparisons and conversions), and basic
// integer/FP32 op latencies.  It also checks that the device si_div, si_log
// and si_neglog_u32 give the same bits as the host.  Every kernel writes only out[global thread] or cyc[0] (in bounds).
//
// Build and run (from the repository root, on a GPU machine):
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -fmad=false \
//        -Xcompiler -ffp-contract=off -o /tmp/latency siminf_gb300/microbench/latency.cu
//   /tmp/latency
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>
#include "../csrc/siminf_stream.h"
#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("ERR %s line %d\n", cudaGetErrorString(e), __LINE__); return 1; } } while (0)

template<int OP>
__global__ void thr(double* out, double a, double b, int n) {
  double x0 = a + threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < n; i++) {
    if (OP == 0) { x0 = __dadd_rn(x0, b); x1 = __dadd_rn(x1, b); x2 = __dadd_rn(x2, b); x3 = __dadd_rn(x3, b); }
    if (OP == 1) { x0 = __fma_rn(x0, a, b); x1 = __fma_rn(x1, a, b); x2 = __fma_rn(x2, a, b); x3 = __fma_rn(x3, a, b); }
    if (OP == 2) { x0 = __dmul_rn(x0, a); x1 = __dmul_rn(x1, a); x2 = __dmul_rn(x2, a); x3 = __dmul_rn(x3, a); }
    if (OP == 3) { x0 = b / x0; x1 = b / x1; x2 = b / x2; x3 = b / x3; }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
template<int OP>
__global__ void thri(unsigned* out, unsigned a, unsigned b, int n) {
  unsigned x0 = a + threadIdx.x, x1 = x0 ^ 1, x2 = x0 ^ 2, x3 = x0 ^ 3;
  for (int i = 0; i < n; i++) {
    if (OP == 0) { x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b; }
    if (OP == 1) { x0 = __umulhi(x0, a) ^ b; x1 = __umulhi(x1, a) ^ b; x2 = __umulhi(x2, a) ^ b; x3 = __umulhi(x3, a) ^ b; }
    if (OP == 2) { float f0 = __int_as_float(x0); f0 = __fmaf_rn(f0, 1.0001f, 0.5f); x0 = __float_as_int(f0);
                   float f1 = __int_as_float(x1); f1 = __fmaf_rn(f1, 1.0001f, 0.5f); x1 = __float_as_int(f1);
                   float f2 = __int_as_float(x2); f2 = __fmaf_rn(f2, 1.0001f, 0.5f); x2 = __float_as_int(f2);
                   float f3 = __int_as_float(x3); f3 = __fmaf_rn(f3, 1.0001f, 0.5f); x3 = __float_as_int(f3); }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
// latency: one dependent chain; only lanes < active do work
template<int OP>
__global__ void lat64(double* out, long long* cyc, double a, double b, int n, int active) {
  if (threadIdx.x >= active) return;
  double x = a + threadIdx.x;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) {
    if (OP == 0) x = __dadd_rn(x, b);
    if (OP == 1) x = __fma_rn(x, a, b);
    if (OP == 3) x = b / x;
  }
  long long t1 = clock64();
  out[threadIdx.x] = x;
  if (threadIdx.x == 0) cyc[0] = t1 - t0;
}

template<int OP> __global__ void latx(double* out, long long* cyc, double a, double b, int n) {
  double x = a + threadIdx.x * 1e-9; int k = threadIdx.x + 3; uint32_t w = 12345 + threadIdx.x;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) {
    if (OP == 0) { x = (double)(k); k = (int)(x * 0.0) + k + 1; }            // I2F.F64 (+F2I)
    if (OP == 1) { k = (x > b) ? k + 1 : k - 1; x = x + 0.0 * k; }           // DSETP chain
    if (OP == 2) { x = b / x; }                                               // DDIV
    if (OP == 3) { x = si_div(b, x); }                                        // soft div
    if (OP == 4) { x = si_log(x + 1.5); }                                     // integer log
    if (OP == 5) { w = w * 1664525u + 1013904223u; x = si_u32_to_uniform_pos(w) + x * 0.0; }
    if (OP == 6) { uint32_t c0=w,c1=1,c2=2,c3=3; si_philox4x32_10(&c0,&c1,&c2,&c3,7,9); w = c0; }
    if (OP == 7) { x = si_neglog_u32(w); w = (uint32_t) si_double_bits(x) * 2654435761u + w; }
  }
  long long t1 = clock64();
  out[threadIdx.x] = x + w + k;
  if (threadIdx.x == 0) cyc[0] = t1 - t0;
}
template<int OP> __global__ void thrx(double* out, double b, int n) {
  double x0 = 1.0 + threadIdx.x * 1e-7, x1 = x0 + 0.25, x2 = x0 + 0.5, x3 = x0 + 0.75;
  for (int i = 0; i < n; i++) {
    if (OP == 2) { x0 = b / x0; x1 = b / x1; x2 = b / x2; x3 = b / x3; }
    if (OP == 3) { x0 = si_div(b, x0); x1 = si_div(b, x1); x2 = si_div(b, x2); x3 = si_div(b, x3); }
    if (OP == 4) { x0 = si_log(x0 + 1.5); x1 = si_log(x1 + 1.5); x2 = si_log(x2 + 1.5); x3 = si_log(x3 + 1.5); }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
__global__ void check_neglog(double* out, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = si_neglog_u32((uint32_t)(i * 255u + (i >> 24)));
}
__global__ void check(const double* a, const double* b, double* q, double* l, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) { q[i] = si_div(a[i], b[i]); l[i] = si_log(a[i] < 0 ? -a[i] : a[i]); }
}
template<int OP> __global__ void lati(unsigned long long* out, long long* cyc, unsigned a, unsigned b, int n) {
  unsigned x = a + threadIdx.x; unsigned long long X = ((unsigned long long)b << 32) | x; float f = 1.0f + threadIdx.x; double d = 1.0 + threadIdx.x;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) {
    if (OP == 0) x = x + b;                             // IADD
    if (OP == 1) x = (x ^ b) | (x >> 3);                // LOP/SHF
    if (OP == 2) x = x * a + b;                         // IMAD
    if (OP == 3) x = __umulhi(x, a) + b;                // IMAD.HI
    if (OP == 4) X = (unsigned long long)(unsigned)X * a + b;   // IMAD.WIDE
    if (OP == 5) X = __umul64hi(X, 0x9E3779B97F4A7C15ULL) + b;  // 64x64 hi
    if (OP == 6) X = X * 0x9E3779B97F4A7C15ULL + b;     // 64-bit mul lo
    if (OP == 7) f = __fmaf_rn(f, 0.999f, 0.5f);        // FFMA
    if (OP == 8) { float r; asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f)); f = r + 1.0f; }  // MUFU.RCP
    if (OP == 9) x = __clzll(X + x) + x;                // FLO/CLZ 64
    if (OP == 10) X = X + ((unsigned long long)x << 7) + (X >> 9);  // 64-bit add/shift
    if (OP == 11) { unsigned long long bits = __double_as_longlong(d); bits ^= b; d = __longlong_as_double(bits | 0x3FF0000000000000ULL); } // MOV f64<->int
  }
  long long t1 = clock64();
  out[threadIdx.x] = x + X + (unsigned long long)f + (unsigned long long)d;
  if (threadIdx.x == 0) cyc[0] = t1 - t0;
}
static uint64_t s_state = 88172645463325252ULL;
static uint64_t xr(void) { s_state ^= s_state << 13; s_state ^= s_state >> 7; s_state ^= s_state << 17; return s_state; }

int main() {
  {

  int dev = 0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, dev));
  printf("GPU %s SMs %d cc %d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
  const int blocks = p.multiProcessorCount * 8, threads = 256, N = 4096;
  double* d; unsigned* u; long long* cyc;
  CK(cudaMalloc(&d, sizeof(double) * blocks * threads));
  CK(cudaMalloc(&u, sizeof(unsigned) * blocks * threads));
  CK(cudaMalloc(&cyc, sizeof(long long)));
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  const char* names[4] = {"DADD", "DFMA", "DMUL", "DDIV"};
  for (int op = 0; op < 4; op++) {
    int n = (op == 3) ? N / 8 : N;
    for (int rep = 0; rep < 2; rep++) {
      cudaEventRecord(e0);
      if (op == 0) thr<0><<<blocks, threads>>>(d, 1.0000001, 1e-9, n);
      if (op == 1) thr<1><<<blocks, threads>>>(d, 0.9999999, 1e-9, n);
      if (op == 2) thr<2><<<blocks, threads>>>(d, 0.9999999, 1e-9, n);
      if (op == 3) thr<3><<<blocks, threads>>>(d, 1.0, 1.0000001, n);
      cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
      float ms; cudaEventElapsedTime(&ms, e0, e1);
      double ops = 4.0 * n * blocks * threads;
      if (rep) printf("%s throughput: %.3f Gop/s (thread-ops), %.2f ms\n", names[op], ops / ms / 1e6, ms);
    }
  }
  const char* inames[3] = {"IMAD32", "UMULHI32", "FFMA32"};
  for (int op = 0; op < 3; op++) {
    for (int rep = 0; rep < 2; rep++) {
      cudaEventRecord(e0);
      if (op == 0) thri<0><<<blocks, threads>>>(u, 1664525u, 1013904223u, N * 4);
      if (op == 1) thri<1><<<blocks, threads>>>(u, 1664525u, 1013904223u, N * 4);
      if (op == 2) thri<2><<<blocks, threads>>>(u, 0x3f800000u, 1u, N * 4);
      cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
      float ms; cudaEventElapsedTime(&ms, e0, e1);
      double ops = 4.0 * N * 4 * blocks * threads;
      if (rep) printf("%s throughput: %.3f Gop/s (thread-ops), %.2f ms\n", inames[op], ops / ms / 1e6, ms);
    }
  }
  int acts[3] = {1, 32, 32};
  for (int op : {0, 1, 3}) for (int k = 0; k < 2; k++) {
    int n = 2048;
    long long c;
    for (int rep = 0; rep < 2; rep++) {
      if (op == 0) lat64<0><<<1, 32>>>(d, cyc, 1.0000001, 1e-9, n, acts[k]);
      if (op == 1) lat64<1><<<1, 32>>>(d, cyc, 0.9999999, 1e-9, n, acts[k]);
      if (op == 3) lat64<3><<<1, 32>>>(d, cyc, 1.0, 1.0000001, n, acts[k]);
      CK(cudaDeviceSynchronize());
      CK(cudaMemcpy(&c, cyc, sizeof(c), cudaMemcpyDeviceToHost));
    }
    printf("%s latency, %d active lanes, 1 warp: %.1f cycles/op\n", names[op], acts[k], (double)c / n);
  }
  // latency with many warps per SM sharing the pipe: 152 blocks x 32 warps, one chain each
  for (int op : {0, 3}) {
    int n = 512; long long c;
    for (int rep = 0; rep < 2; rep++) {
      if (op == 0) lat64<0><<<p.multiProcessorCount, 1024>>>(d, cyc, 1.0000001, 1e-9, n, 1024);
      if (op == 3) lat64<3><<<p.multiProcessorCount, 1024>>>(d, cyc, 1.0, 1.0000001, n, 1024);
      CK(cudaDeviceSynchronize());
      CK(cudaMemcpy(&c, cyc, sizeof(c), cudaMemcpyDeviceToHost));
    }
    printf("%s per-op cycles, 32 warps/SM one chain each: %.1f cycles/op\n", names[op], (double)c / n);
  }
  printf("done\n");
    }
  int bad = 0;
  {

  double* d2; long long* cyc2; CK(cudaMalloc(&d2, sizeof(double) * 152 * 8 * 256)); CK(cudaMalloc(&cyc2, 8));
  const char* nm[8] = {"I2F.F64+F2I", "DSETP-select", "DDIV", "si_div", "si_log", "uniform_pos", "philox4x32-10", "si_neglog_u32"};
  for (int op = 0; op < 8; op++) {
    long long c = 0; int n = 512;
    for (int rep = 0; rep < 2; rep++) {
      switch (op) { case 0: latx<0><<<1,32>>>(d2,cyc2,1.1,1.3,n); break; case 1: latx<1><<<1,32>>>(d2,cyc2,1.1,1.3,n); break;
        case 2: latx<2><<<1,32>>>(d2,cyc2,1.1,1.3,n); break; case 3: latx<3><<<1,32>>>(d2,cyc2,1.1,1.3,n); break;
        case 4: latx<4><<<1,32>>>(d2,cyc2,1.1,1.3,n); break; case 5: latx<5><<<1,32>>>(d2,cyc2,1.1,1.3,n); break;
        case 6: latx<6><<<1,32>>>(d2,cyc2,1.1,1.3,n); break; case 7: latx<7><<<1,32>>>(d2,cyc2,1.1,1.3,n); break; }
      CK(cudaDeviceSynchronize()); CK(cudaMemcpy(&c, cyc2, 8, cudaMemcpyDeviceToHost));
    }
    printf("latency %-14s %.1f cycles/op\n", nm[op], (double)c / n);
  }
  cudaEvent_t f0, f1; cudaEventCreate(&f0); cudaEventCreate(&f1);
  for (int op = 2; op <= 4; op++) {
    int n = 256; float ms = 0;
    for (int rep = 0; rep < 2; rep++) {
      cudaEventRecord(f0);
      if (op == 2) thrx<2><<<152*8,256>>>(d2, 1.3, n); if (op == 3) thrx<3><<<152*8,256>>>(d2, 1.3, n); if (op == 4) thrx<4><<<152*8,256>>>(d2, 1.3, n);
      cudaEventRecord(f1); CK(cudaEventSynchronize(f1)); cudaEventElapsedTime(&ms, f0, f1);
    }
    printf("throughput %-8s %.1f Gop/s\n", nm[op], 4.0 * n * 152 * 8 * 256 / ms / 1e6);
  }
  // device-vs-host bit equality of si_div and si_log
  const long N = 1 << 24; double *ha = (double*)malloc(N*8), *hb = (double*)malloc(N*8), *hq = (double*)malloc(N*8), *hl = (double*)malloc(N*8);
  for (long i = 0; i < N; i++) { uint64_t r = xr(), q = xr(); int m = i % 6;
    if (m == 0) { ha[i] = si_bits_double(r & 0x7FFFFFFFFFFFFFFFULL); hb[i] = si_bits_double(q); }
    else if (m == 1) { ha[i] = (double)(r % 100000) + 1; hb[i] = (double)(q % 1000) + 0.5; }
    else if (m == 2) { ha[i] = si_bits_double(0x3FF0000000000000ULL | (r & 0xFFFFFFFFFFFFFULL)); hb[i] = si_bits_double(0x3FF0000000000000ULL | ((r + (q & 3)) & 0xFFFFFFFFFFFFFULL)); }
    else if (m == 3) { ha[i] = si_bits_double(0x3FF0000000000000ULL | (r & 0xFFFFFFFFFFFFFULL)); hb[i] = si_bits_double(0x4010000000000000ULL | (q & 0xFF)); }
    else if (m == 4) { ha[i] = si_bits_double(0x3FFFFFFFFFFFFFFFULL - (r & 0xFFFF)); hb[i] = si_bits_double(0x3FFFFFFFFFFFFFFFULL - (q & 0xFF)); }
    else { ha[i] = si_bits_double(0x0010000000000000ULL | (r & 0x3FFFFFFFFFFFFFULL)); hb[i] = si_bits_double(0x7FE0000000000000ULL - (q & 0x00FFFFFFFFFFFFFFULL)); } }
  double *da, *db, *dq, *dl; CK(cudaMalloc(&da, N*8)); CK(cudaMalloc(&db, N*8)); CK(cudaMalloc(&dq, N*8)); CK(cudaMalloc(&dl, N*8));
  CK(cudaMemcpy(da, ha, N*8, cudaMemcpyHostToDevice)); CK(cudaMemcpy(db, hb, N*8, cudaMemcpyHostToDevice));
  check<<<(N+255)/256, 256>>>(da, db, dq, dl, N); CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(hq, dq, N*8, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(hl, dl, N*8, cudaMemcpyDeviceToHost));
  long bq = 0, bl = 0;
  for (long i = 0; i < N; i++) {
    double q = ha[i] / hb[i]; if (si_double_bits(q) != si_double_bits(hq[i]) && !(q != q && hq[i] != hq[i])) bq++;
    double l = si_log(ha[i] < 0 ? -ha[i] : ha[i]); if (si_double_bits(l) != si_double_bits(hl[i]) && !(l != l && hl[i] != hl[i])) bl++; }
  printf("device si_div vs host division mismatches: %ld of %ld\n", bq, N);
  printf("device si_log vs host si_log mismatches: %ld of %ld\n", bl, N);
  check_neglog<<<(N+255)/256, 256>>>(dl, N); CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(hl, dl, N*8, cudaMemcpyDeviceToHost));
  long bn = 0;
  for (long i = 0; i < N; i++)
    if (si_double_bits(si_neglog_u32((uint32_t)(i * 255u + (i >> 24)))) != si_double_bits(hl[i])) bn++;
  printf("device si_neglog_u32 vs host mismatches: %ld of %ld\n", bn, N);
      bad = (bq || bl || bn);
  }
  {

  unsigned long long* o; long long* c; cudaMalloc(&o, 32 * 8); cudaMalloc(&c, 8);
  const char* nm[12] = {"IADD", "LOP+SHF", "IMAD", "IMAD.HI", "IMAD.WIDE", "umul64hi", "mul64lo", "FFMA", "MUFU.RCP+FADD", "CLZ64", "add64+shift64", "f64<->bits"};
  for (int op = 0; op < 12; op++) {
    long long cc = 0; int n = 1024;
    for (int r = 0; r < 2; r++) {
      switch (op) {
        case 0: lati<0><<<1,32>>>(o,c,3,5,n); break; case 1: lati<1><<<1,32>>>(o,c,3,5,n); break;
        case 2: lati<2><<<1,32>>>(o,c,3,5,n); break; case 3: lati<3><<<1,32>>>(o,c,3,5,n); break;
        case 4: lati<4><<<1,32>>>(o,c,3,5,n); break; case 5: lati<5><<<1,32>>>(o,c,3,5,n); break;
        case 6: lati<6><<<1,32>>>(o,c,3,5,n); break; case 7: lati<7><<<1,32>>>(o,c,3,5,n); break;
        case 8: lati<8><<<1,32>>>(o,c,3,5,n); break; case 9: lati<9><<<1,32>>>(o,c,3,5,n); break;
        case 10: lati<10><<<1,32>>>(o,c,3,5,n); break; case 11: lati<11><<<1,32>>>(o,c,3,5,n); break; }
      cudaDeviceSynchronize(); cudaMemcpy(&cc, c, 8, cudaMemcpyDeviceToHost);
    }
    printf("latency %-14s %.1f cycles/op\n", nm[op], (double)cc / n);
  }
    }
  return bad ? 2 : 0;
}
