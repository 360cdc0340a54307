// Declarations of the per-class kernel launchers (explicitly instantiated in
// the gnlse_inst_*.cu translation units) and the table of supported classes.
#pragma once
#include <cuda_runtime.h>

#include "gnlse_dd.cuh"
#include "gnlse_types.h"

namespace gnlse {

// kernel of the RK4IP stage loop (RK4IP, ARK4IP, ss_sym_rk4)
template <class R, int LOGM, int C, bool XS>
cudaError_t launch_class(const KParams& kp, int n_clusters, cudaStream_t stream);
// kernel of the exponential split steps (ss_symmetric, ss_simple, ss_reduced)
template <class R, int LOGM, int C, bool XS>
cudaError_t launch_class_ss(const KParams& kp, int n_clusters, cudaStream_t stream);

// (precision, log2 M, C) classes compiled into the library.
#ifdef GNLSE_ENSEMBLE_SUBSET
// tuning builds: only the FP32 classes of the ensemble benchmark
#define GNLSE_CLASSES_F32(X) X(float, 12, 1)
#define GNLSE_CLASSES_F64(X)
#define GNLSE_CLASSES_DF(X) X(ddf, 12, 1) X(ddf, 12, 2) X(ddf, 12, 4) X(ddf, 11, 4) X(ddf, 11, 8)
#define GNLSE_CLASSES_MIX(X) \
  X(float, 12, 1) X(float, 12, 2) X(float, 12, 4) X(float, 11, 2) X(float, 11, 4) X(float, 11, 8) \
  X(float, 13, 1) X(float, 13, 2)
#else
// (complex64 clusters of 256- and 512-point slices are not offered: their 64-thread
// CTAs leave half the threads idle in every radix pass, compile to kernels that
// spill ~4 KB per thread, and the 2 x 512 one faulted on a GB300; a 1024-point
// complex64 grid runs in one CTA.)
#define GNLSE_CLASSES_F32(X) \
  X(float, 8, 1) X(float, 9, 1) X(float, 10, 1) X(float, 11, 1) X(float, 12, 1) X(float, 13, 1) \
  X(float, 10, 2) X(float, 12, 2) X(float, 13, 2) \
  X(float, 12, 4) X(float, 13, 4) X(float, 12, 8) X(float, 13, 8)
#define GNLSE_CLASSES_F64(X) \
  X(double, 8, 1) X(double, 9, 1) X(double, 10, 1) X(double, 11, 1) X(double, 12, 1) \
  X(double, 8, 2) X(double, 9, 2) X(double, 10, 2) X(double, 11, 2) X(double, 12, 2) \
  X(double, 8, 4) X(double, 12, 4) X(double, 12, 8) X(double, 12, 16)
// double-float classes: ~48-bit transforms, nonlinear term and state on FP32 instructions
#define GNLSE_CLASSES_DF(X) \
  X(ddf, 10, 1) X(ddf, 11, 1) X(ddf, 12, 1) X(ddf, 11, 2) X(ddf, 12, 2) \
  X(ddf, 11, 4) X(ddf, 12, 4) X(ddf, 11, 8) X(ddf, 12, 8) X(ddf, 12, 16)
// extended-state (mixed precision) classes: complex64 transforms
#define GNLSE_CLASSES_MIX(X) \
  X(float, 8, 1) X(float, 9, 1) X(float, 10, 1) X(float, 11, 1) X(float, 12, 1) \
  X(float, 9, 2) X(float, 12, 2) X(float, 8, 4) X(float, 12, 4) X(float, 12, 8) X(float, 13, 8) \
  X(float, 11, 2) X(float, 11, 4) X(float, 11, 8) X(float, 13, 1) X(float, 13, 2)
#endif

}  // namespace gnlse
