// double instances of the pass launchers (the plain FP64 path)
#define XPFC_T double
#define XPFC_XTAG f64
#include "xpfc_launch.inc"
