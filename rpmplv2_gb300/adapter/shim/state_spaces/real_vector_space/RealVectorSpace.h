// RealVectorSpace.h -- RPMPLv2's base::RealVectorSpace
// (include/state_spaces/real_vector_space/RealVectorSpace.h:17-52) reduced to
// the collision and distance path: its two constructors (with and without the
// robot and environment) and the same four virtuals, whose CPU
// implementations (RealVectorSpace.cpp:261-446) RealVectorSpaceGPU replaces.
#pragma once
#include "../StateSpace.h"
#include "RealVectorSpaceState.h"

namespace base {

class RealVectorSpace : public StateSpace {
public:
    RealVectorSpace(size_t num_dimensions_) : StateSpace(num_dimensions_) {}
    RealVectorSpace(size_t num_dimensions_, const std::shared_ptr<robots::AbstractRobot> robot_,
                    const std::shared_ptr<env::Environment> env_)
        : StateSpace(num_dimensions_, robot_, env_) {}
    virtual ~RealVectorSpace() {}

    bool isValid(const std::shared_ptr<base::State> q1, const std::shared_ptr<base::State> q2) override = 0;
    bool isValid(const std::shared_ptr<base::State> q) override = 0;
    float computeDistance(const std::shared_ptr<base::State> q, bool compute_again = false) override = 0;
    float computeDistanceUnderestimation(const std::shared_ptr<base::State> q,
                                         const std::shared_ptr<std::vector<Eigen::MatrixXf>> nearest_points) override = 0;
};

}  // namespace base
