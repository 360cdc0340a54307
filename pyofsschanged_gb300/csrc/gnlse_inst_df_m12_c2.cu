// Kernel instantiation: double-float, M = 2^12 points per CTA, cluster of 2.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(gnlse::ddf, 12, 2)
