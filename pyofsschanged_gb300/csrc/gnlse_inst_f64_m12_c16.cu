// Kernel instantiation: double, M = 2^12 points per CTA, cluster of 16.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(double, 12, 16)
