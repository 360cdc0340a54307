// Kernel instantiation: float, M = 2^9 points per CTA, cluster of 1.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(float, 9, 1)
