// Kernel instantiation: double-float, M = 2^10 points per CTA, cluster of 1.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(gnlse::ddf, 10, 1)
