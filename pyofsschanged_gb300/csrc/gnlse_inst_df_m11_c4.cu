// Kernel instantiation: double-float, M = 2^11 points per CTA, cluster of 4.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(gnlse::ddf, 11, 4)
