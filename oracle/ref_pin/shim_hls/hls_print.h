// Stand-in for the Xilinx HLS print header (nothing of it is used).
#ifndef REF_PIN_HLS_PRINT_H
#define REF_PIN_HLS_PRINT_H
#endif
