// RealVectorSpaceState.h -- RPMPLv2's concrete state of a RealVectorSpace
// (include/state_spaces/real_vector_space/RealVectorSpaceState.h).
#pragma once
#include "../State.h"

namespace base {

class RealVectorSpaceState : public State {
public:
    RealVectorSpaceState(const Eigen::VectorXf &coord_) : State(coord_) {}
    ~RealVectorSpaceState() {}
};

}  // namespace base
