// Stand-in for the Xilinx AXI-stream side-channel header: only named in typedefs.
#ifndef REF_PIN_AP_AXI_SDATA_H
#define REF_PIN_AP_AXI_SDATA_H
#include "ap_int.h"
template <int D, int U, int TI, int TD> struct ap_axiu {};
#endif
