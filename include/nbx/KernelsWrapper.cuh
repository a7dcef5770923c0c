// KernelsWrapper.cuh -- drop-in for the reference's include/KernelsWrapper.cuh
// (3D/CUDA/CUDA_NBody/include/KernelsWrapper.cuh:15-50): the seven phase
// methods over libnbx (nbx::KernelsWrapper) in the global namespace.
#pragma once

#include "barnes_hut.hpp"

using nbx::KernelsWrapper;
