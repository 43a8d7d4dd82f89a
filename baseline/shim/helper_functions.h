/* Stand-in for cuda-samples' helper_functions.h: LC2500/XPFC_CUDA includes it
   (globals.cuh:12) but uses nothing from it. */
#pragma once
