// Status codes shared by host and device code (the public values are declared
// in phpc_gemm.h; this header only pulls them in for the kernels).
#pragma once
#include "phpc_gemm.h"
