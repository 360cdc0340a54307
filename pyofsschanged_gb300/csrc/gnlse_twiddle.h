// Layout of the per-pass twiddle table of the M-point Stockham transform.
//
// Pass p (sub-transform size Ns = R^p, radix RAD) multiplies input r of
// butterfly k (k < Ns) by W_{Ns*RAD}^{r k} = W_M^{r k M/(Ns RAD)}.  The table
// holds one row of RAD entries per (pass, k) -- entry r of the row is that
// twiddle (r = 0 holds W^0) -- so a thread reads its butterfly's twiddles as
// one contiguous, 128-byte aligned row instead of RAD-1 scattered entries.
// Shared by the host table builders and the device passes.
#pragma once

#ifndef GNLSE_RADIX_BITS
#define GNLSE_RADIX_BITS 4
#endif
// double-float plans: radix-8 passes, 8 points per thread (a radix-16 butterfly of
// 16-byte double-float values needs the whole register file of a 256-thread CTA)
#ifndef GNLSE_DF_RADIX_BITS
#define GNLSE_DF_RADIX_BITS 3
#endif

#if defined(__CUDACC__)
#define GNLSE_HD __host__ __device__
#else
#define GNLSE_HD
#endif

namespace gnlse {

// first entry of the rows of pass p (main radix R = 2^rb passes, then the
// final radix-2^(logm % rb) pass as p = logm / rb)
GNLSE_HD constexpr int twp_offset(int logm, int rb, int p) {
  int off = 0, ns = 1;
  for (int q = 0; q < p; ++q) {
    const int rad = q < logm / rb ? (1 << rb) : (1 << (logm % rb));
    off += ns * rad;
    ns *= rad;
  }
  return off;
}

GNLSE_HD constexpr int twp_size(int logm, int rb) {
  return twp_offset(logm, rb, logm / rb + ((logm % rb) ? 1 : 0));
}

// exponent j of W_M^j stored at entry e
GNLSE_HD inline int twp_exponent(int logm, int rb, int e) {
  const int M = 1 << logm;
  const int np = logm / rb + ((logm % rb) ? 1 : 0);
  int off = 0, ns = 1;
  for (int p = 0; p < np; ++p) {
    const int rad = p < logm / rb ? (1 << rb) : (1 << (logm % rb));
    if (e < off + ns * rad) {
      const int k = (e - off) / rad, r = (e - off) % rad;
      return r * k * (M / (ns * rad));
    }
    off += ns * rad;
    ns *= rad;
  }
  return 0;
}

}  // namespace gnlse
