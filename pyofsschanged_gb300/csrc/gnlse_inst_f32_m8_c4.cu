// Kernel instantiation: float, M = 2^8 points per CTA, cluster of 4.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(float, 8, 4)
