/* Stand-in for the CUDA samples' helper_functions.h (gpu4snn.cu:38); nothing from it is used. */
#pragma once
