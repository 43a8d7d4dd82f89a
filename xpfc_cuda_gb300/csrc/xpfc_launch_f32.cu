// float instances of the pass launchers (the mixed-precision path)
#define XPFC_T float
#define XPFC_XTAG f32
#define XPFC_COMMON
#include "xpfc_launch.inc"
