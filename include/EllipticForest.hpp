// Umbrella header of the C++ drop-in for EllipticForest's HPS path (the reference's
// src/EllipticForest.hpp).  Drivers written against the reference compile with -I<repo>/include and
// link against ellipticforest_gb300/libellipticforest_gb300.so.
#pragma once

#include "EllipticForest/Core.hpp"
#include "EllipticForest/FiniteVolume.hpp"
#include "EllipticForest/HPSAlgorithm.hpp"
#include "EllipticForest/Mesh.hpp"
