// Kernel instantiation: double, M = 2^10 points per CTA, cluster of 2.
#include "gnlse_inst.inc"
GNLSE_INSTANTIATE(double, 10, 2)
