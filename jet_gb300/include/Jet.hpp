// Umbrella header of the GB300 Jet host API.
#pragma once

#include "jet/Abort.hpp"
#if __has_include(<cuComplex.h>)
#include "jet/CudaTensor.hpp"
#endif
#include "jet/PathInfo.hpp"
#include "jet/SlicedContractor.hpp"
#include "jet/TaskBasedContractor.hpp"
#include "jet/Tensor.hpp"
#include "jet/TensorNetwork.hpp"
#include "jet/Utilities.hpp"
#include "jet/permute/Permuter.hpp"
