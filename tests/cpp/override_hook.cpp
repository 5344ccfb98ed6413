// A reference-style subclass that overrides a per-node hook of HPSAlgorithm.  The drop-in runs every
// tree level as grouped GPU kernels and never calls the hooks per node, so it declares them final:
// this file must NOT compile (the compile-fail test expects "final" in the diagnostic).
#include <EllipticForest.hpp>
#include <Patches/FiniteVolume/FiniteVolume.hpp>

namespace ef = EllipticForest;
using Base = ef::HPSAlgorithm<ef::FiniteVolumeGrid, ef::FiniteVolumeSolver, ef::FiniteVolumePatch, double>;

class MyHPS : public Base {
public:
    using Base::Base;
    void merge4to1(ef::FiniteVolumePatch& tau, ef::FiniteVolumePatch& alpha, ef::FiniteVolumePatch& beta,
                   ef::FiniteVolumePatch& gamma, ef::FiniteVolumePatch& omega) override {}
};

int main() { return 0; }
