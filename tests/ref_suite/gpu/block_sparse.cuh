// Include-path stand-in for the reference's "gpu/block_sparse.cuh", so that
// the reference's own GPU test sources compile, unchanged, against the
// drop-in class.  Like the reference header it brings in cuBLAS's declarations
// (callers create the handle that contract() takes) and the reference's CPU
// tensors (its tests use torque::DenseTensor as the expected value), and a
// DEBUG(n) marker print.
#pragma once
#include <cublas_v2.h>

#include <cstdio>

#include "tensor/block_sparse.h"
#include "torque_gb300/block_sparse.hpp"

// The reference header's helpers also give its programs a DEBUG(n) marker
// print; its benchmarks use it.
#ifndef DEBUG
#define DEBUG(n) std::printf("marker %d\n", (int)(n));
#endif
