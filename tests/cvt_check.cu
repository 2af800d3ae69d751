// GPU check of the integer-pipe conversions d2f_alu / f2d_alu of lh_internal.cuh against the
// hardware conversions (tests/test_gpu_cvt.py builds and runs it). Inputs: ties between two
// floats with an even and an odd lower neighbour, carries of the rounding into the exponent,
// the overflow edge around FLT_MAX + half an ulp, the smallest normal and the subnormal range,
// signed zeros, infinities, NaN, and random doubles over every float exponent.
// Contract checked: d2f_alu(x) is bit-identical to __double2float_rn(x) for every x with
// |x| >= 2^-126 (normal results, the carry into the exponent, rounding up to infinity), a NaN
// for a NaN, and a zero of x's sign for |x| < 2^-126 (where the hardware gives a subnormal,
// a zero, or FLT_MIN for the half ulp just below it).
// f2d_alu(f) is bit-identical to (double)f for every non-subnormal float, and a signed zero
// for subnormal floats.
// Output: one line "d2f <checked> <mismatches> f2d <checked> <mismatches>".
#include "../rnl_multiblock_nofft_gb300/csrc/lh_internal.cuh"

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

__global__ void k_d2f(const double *x, unsigned *alu, unsigned *hw, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  alu[i] = __float_as_uint(d2f_alu(x[i]));
  hw[i] = __float_as_uint(__double2float_rn(x[i]));
}
__global__ void k_f2d(const float *x, unsigned long long *alu, unsigned long long *hw, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  alu[i] = (unsigned long long)__double_as_longlong(f2d_alu(x[i]));
  hw[i] = (unsigned long long)__double_as_longlong((double)x[i]);
}

static double from_bits(unsigned long long b) { double d; memcpy(&d, &b, 8); return d; }
static unsigned long long bits(double d) { unsigned long long b; memcpy(&b, &d, 8); return b; }
static float f_from_bits(unsigned b) { float f; memcpy(&f, &b, 4); return f; }

#define CKC(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_)); return 2; } } while (0)

int main() {
  std::vector<double> xd;
  std::mt19937_64 rng(12345);
  // ties and near-ties around float values with even and odd mantissas, every exponent
  for (int e = -126; e <= 127; ++e) {
    for (unsigned m : {0u, 1u, 2u, 3u, 0x3ffffeu, 0x7ffffeu, 0x7fffffu, 0x400000u, 0x123457u}) {
      const double f = ldexp(1.0 + (double)m / 8388608.0, e);  // a float value
      const double ulp = ldexp(1.0, e - 23);
      for (double o : {0.0, 0.5, -0.5, 0.25, 0.75}) {
        const double x = f + o * ulp;
        for (double s : {1.0, -1.0}) {
          xd.push_back(s * x);
          xd.push_back(from_bits(bits(s * x) + 1));  // one double ulp above
          xd.push_back(from_bits(bits(s * x) - 1));  // and below
        }
      }
    }
  }
  // the overflow edge: FLT_MAX, FLT_MAX + half a float ulp (rounds to inf), just below it
  const double fmax = (double)FLT_MAX, half = ldexp(1.0, 127 - 24);
  const std::vector<double> edge = {fmax, fmax + half, from_bits(bits(fmax + half) - 1),
                                    from_bits(bits(fmax + half) + 1), 2.0 * fmax, ldexp(1.0, 128), 1e300,
                                    (double)INFINITY};
  for (double x : edge) {
    xd.push_back(x);
    xd.push_back(-x);
  }
  // zeros, the smallest normal, the subnormal range, NaN
  const std::vector<double> small = {0.0, -0.0, (double)FLT_MIN, ldexp(1.0, -127), ldexp(1.0, -140),
                                     ldexp(1.0, -149), ldexp(1.0, -150), 1e-300, 4.9e-324,
                                     (double)FLT_MIN * (1.0 - ldexp(1.0, -30))};
  for (double x : small) { xd.push_back(x); xd.push_back(-x); }
  xd.push_back(NAN);
  xd.push_back(-NAN);
  // random doubles over the float exponent range and random bit patterns
  for (int i = 0; i < 200000; ++i) {
    std::uniform_real_distribution<double> u(-130.0, 130.0);
    xd.push_back(ldexp(std::uniform_real_distribution<double>(-1.0, 1.0)(rng), (int)u(rng)));
    xd.push_back(from_bits(rng()));
  }
  std::vector<float> xf;
  for (unsigned b : {0u, 0x80000000u, 0x00800000u, 0x80800000u, 0x007fffffu, 0x00000001u, 0x7f7fffffu, 0xff7fffffu,
                     0x7f800000u, 0xff800000u, 0x7fc00000u, 0x7f800001u, 0x3f800000u})
    xf.push_back(f_from_bits(b));
  for (int i = 0; i < 400000; ++i) xf.push_back(f_from_bits((unsigned)rng()));

  const int nd = (int)xd.size(), nf = (int)xf.size();
  double *dx; unsigned *da, *dh; float *fx; unsigned long long *fa, *fh;
  CKC(cudaMalloc(&dx, sizeof(double) * nd));
  CKC(cudaMalloc(&da, sizeof(unsigned) * nd));
  CKC(cudaMalloc(&dh, sizeof(unsigned) * nd));
  CKC(cudaMalloc(&fx, sizeof(float) * nf));
  CKC(cudaMalloc(&fa, sizeof(unsigned long long) * nf));
  CKC(cudaMalloc(&fh, sizeof(unsigned long long) * nf));
  CKC(cudaMemcpy(dx, xd.data(), sizeof(double) * nd, cudaMemcpyHostToDevice));
  CKC(cudaMemcpy(fx, xf.data(), sizeof(float) * nf, cudaMemcpyHostToDevice));
  k_d2f<<<(nd + 255) / 256, 256>>>(dx, da, dh, nd);
  k_f2d<<<(nf + 255) / 256, 256>>>(fx, fa, fh, nf);
  CKC(cudaGetLastError());
  CKC(cudaDeviceSynchronize());
  std::vector<unsigned> ra(nd), rh(nd);
  std::vector<unsigned long long> qa(nf), qh(nf);
  CKC(cudaMemcpy(ra.data(), da, sizeof(unsigned) * nd, cudaMemcpyDeviceToHost));
  CKC(cudaMemcpy(rh.data(), dh, sizeof(unsigned) * nd, cudaMemcpyDeviceToHost));
  CKC(cudaMemcpy(qa.data(), fa, sizeof(unsigned long long) * nf, cudaMemcpyDeviceToHost));
  CKC(cudaMemcpy(qh.data(), fh, sizeof(unsigned long long) * nf, cudaMemcpyDeviceToHost));
  long bad_d = 0, bad_f = 0;
  for (int i = 0; i < nd; ++i) {
    const unsigned h = rh[i], a = ra[i], sign = h & 0x80000000u;
    const unsigned mag = h & 0x7fffffffu;
    bool ok;
    if (mag > 0x7f800000u) ok = (a & 0x7fffffffu) > 0x7f800000u;  // NaN in, NaN out
    else if (fabs(xd[i]) < (double)FLT_MIN) ok = (a == sign);     // below the normal range: signed zero
    else ok = (a == h);
    if (!ok) { if (bad_d < 8) fprintf(stderr, "d2f %.17g: alu %08x hw %08x\n", xd[i], a, h); ++bad_d; }
  }
  for (int i = 0; i < nf; ++i) {
    unsigned b; memcpy(&b, &xf[i], 4);
    const unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    bool ok;
    if (e == 255u && m) ok = ((qa[i] >> 52) & 0x7ffu) == 0x7ffu && (qa[i] & 0xfffffffffffffull);
    else if (e == 0u) ok = qa[i] == ((unsigned long long)(b & 0x80000000u) << 32);
    else ok = qa[i] == qh[i];
    if (!ok) { if (bad_f < 8) fprintf(stderr, "f2d %08x: alu %016llx hw %016llx\n", b, qa[i], qh[i]); ++bad_f; }
  }
  printf("d2f %d %ld f2d %d %ld\n", nd, bad_d, nf, bad_f);
  return 0;
}
