/* Stand-in for cuda-samples' helper_functions.h (absent from this image). */
#pragma once
