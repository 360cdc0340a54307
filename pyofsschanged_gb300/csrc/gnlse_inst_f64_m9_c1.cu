// Kernel instantiation: double, M = 2^9 points per CTA, cluster of 1.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(double, 9, 1)
