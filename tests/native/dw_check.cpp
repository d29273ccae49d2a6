// Error of the double-word operations of woo_gb300/csrc/wdem_dw.cuh against long double, on seeded values in
// the ranges of the contact law (magnitudes 1e-12 .. 1e12).  Prints the largest relative error of each
// operation in units of u^2 = 2^-48, and the count of conversions that left the words unnormalised.
#include "../../woo_gb300/csrc/wdem_dw.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace wdem;
typedef long double LD;
static LD val(dwf x) { return (LD)x.h + (LD)x.l; }
static double rel(LD x, LD ref) { return ref == 0 ? (double)fabsl(x) : (double)fabsl((x - ref) / ref); }

int main() {
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<double> U(-1, 1), E(-12, 12);
  double worst[7] = {0, 0, 0, 0, 0, 0, 0};
  long unnormalised = 0, roundtrip = 0;
  for (int it = 0; it < 400000; it++) {
    const double a = U(g) * std::pow(10.0, E(g));
    double b = U(g) * std::pow(10.0, E(g) * 0.3);
    if (it % 3 == 0) b = a * (1 + 1e-3 * U(g));
    const dwf A = dwFrom(a), B = dwFrom(b);
    if (A.l != 0 && fabsf(A.l) > std::ldexp(fabsf(A.h), -24) * 1.0000001f) unnormalised++;
    if (dwTo(A) != (double)val(A)) roundtrip++;
    worst[0] = std::fmax(worst[0], rel(val(A), a));
    const LD s = val(A) + val(B);
    if (fabsl(s) > 1e-6L * (fabsl(val(A)) + fabsl(val(B)))) worst[1] = std::fmax(worst[1], rel(val(dwAdd(A, B)), s));
    worst[2] = std::fmax(worst[2], rel(val(dwMul(A, B)), val(A) * val(B)));
    worst[3] = std::fmax(worst[3], rel(val(dwDiv(A, B)), val(A) / val(B)));
    const dwf Aa = dwAbs(A);
    worst[4] = std::fmax(worst[4], rel(val(dwSqrt(Aa)), sqrtl(val(Aa))));
    const float f = (float)b;
    worst[5] = std::fmax(worst[5], rel(val(dwMulF(A, f)), val(A) * (LD)f));
    const LD sf = val(A) + (LD)f;
    if (fabsl(sf) > 1e-6L * (fabsl(val(A)) + fabsl((LD)f))) worst[6] = std::fmax(worst[6], rel(val(dwAddF(A, f)), sf));
  }
  const double u2 = std::ldexp(1.0, -48);
  printf("from %.3f\nadd %.3f\nmul %.3f\ndiv %.3f\nsqrt %.3f\nmulF %.3f\naddF %.3f\nunnormalised %ld\nroundtrip %ld\n",
         worst[0] / u2, worst[1] / u2, worst[2] / u2, worst[3] / u2, worst[4] / u2, worst[5] / u2, worst[6] / u2,
         unnormalised, roundtrip);
  return 0;
}
