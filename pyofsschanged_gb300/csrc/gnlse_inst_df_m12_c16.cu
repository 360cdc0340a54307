// Kernel instantiation: double-float, M = 2^12 points per CTA, cluster of 16.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(gnlse::ddf, 12, 16)
