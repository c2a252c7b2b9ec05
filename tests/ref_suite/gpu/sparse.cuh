// Include-path stand-in for the reference's "gpu/sparse.cuh" (see
// block_sparse.cuh beside it): cuBLAS's declarations and the drop-in
// element-sparse class.
#pragma once
#include <cublas_v2.h>

#include "torque_gb300/sparse.hpp"
