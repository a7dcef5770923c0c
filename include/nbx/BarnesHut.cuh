// BarnesHut.cuh -- drop-in for the reference's include/BarnesHut.cuh
// (3D/CUDA/CUDA_NBody/include/BarnesHut.cuh:18-127): the libnbx host class
// nbx::BarnesHut in the global namespace, constructed from the application's
// SimulationParameters (its Constants.h, included before this header, as the
// reference's main.cu does).
#pragma once

#include "barnes_hut.hpp"

using nbx::BarnesHut;
