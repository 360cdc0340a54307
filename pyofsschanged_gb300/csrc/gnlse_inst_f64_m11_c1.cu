// Kernel instantiation: double, M = 2^11 points per CTA, cluster of 1.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(double, 11, 1)
