// Kernel instantiation: float, M = 2^10 points per CTA, cluster of 2.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(float, 10, 2)
