// Stand-in for the Xilinx HLS fixed-point header: only named in typedefs.
#ifndef REF_PIN_AP_FIXED_H
#define REF_PIN_AP_FIXED_H
#include "ap_int.h"
template <int W, int I> struct ap_fixed {};
#endif
