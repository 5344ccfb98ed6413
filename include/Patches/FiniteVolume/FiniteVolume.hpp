// Same include path as the reference's src/Patches/FiniteVolume/FiniteVolume.hpp.
#pragma once

#include "../../EllipticForest/FiniteVolume.hpp"
#include "../../EllipticForest/Mesh.hpp"
