// Kernel instantiation: extended-state complex64, M = 2^13 points per CTA, cluster of 2.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE_MIX(13, 2)
