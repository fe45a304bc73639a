// Drop-in header with the reference's name (lsq_transformer.hpp): the GPU
// implementation lives in zest_gpu.hpp.
#pragma once
#include "zest_gpu.hpp"
