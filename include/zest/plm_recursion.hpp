// Drop-in header with the reference's name (plm_recursion.hpp): the GPU
// implementation of the whole transform and rotation interface lives in
// zest_gpu.hpp.
#pragma once
#include "zest_gpu.hpp"
