// double instances of the pass launchers (the plain FP64 path)
#define XPFC_T double
#include "xpfc_launch.inc"
