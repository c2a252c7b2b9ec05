// Include-path stand-in for the reference's "gpu/dense.cuh" (see
// block_sparse.cuh beside it): cuBLAS's declarations, the reference's index
// helpers (util/space.h, which its header includes) and the drop-in dense
// class.
#pragma once
#include <cublas_v2.h>

#include "util/space.h"

#include "torque_gb300/dense.hpp"
