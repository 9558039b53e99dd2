// StateSpace.h -- the collision and distance interface of RPMPLv2's
// base::StateSpace (include/state_spaces/StateSpace.h:16-57), with the same
// signatures and the same public members: num_dimensions and the space's
// robot and environment (StateSpace.h:20-21), which planners dereference
// (DRGBT.cpp:15, 31; MotionValidity.cpp:12-15, 39-42).  Planners call the four
// collision and distance virtuals; nothing else of the state space is needed
// by the path.
#pragma once
#include <memory>
#include <vector>

#include <environments/Environment.h>
#include <robots/AbstractRobot.h>

#include "State.h"

namespace base {

class StateSpace {
public:
    size_t num_dimensions;
    std::shared_ptr<robots::AbstractRobot> robot;
    std::shared_ptr<env::Environment> env;

    StateSpace(size_t num_dimensions_) : num_dimensions(num_dimensions_) {}
    StateSpace(size_t num_dimensions_, const std::shared_ptr<robots::AbstractRobot> robot_,
               const std::shared_ptr<env::Environment> env_)
        : num_dimensions(num_dimensions_), robot(robot_), env(env_) {}
    virtual ~StateSpace() {}
    inline size_t getNumDimensions() { return num_dimensions; }

    virtual bool isValid(const std::shared_ptr<base::State> q) = 0;
    virtual bool isValid(const std::shared_ptr<base::State> q1, const std::shared_ptr<base::State> q2) = 0;
    virtual float computeDistance(const std::shared_ptr<base::State> q, bool compute_again = false) = 0;
    virtual float computeDistanceUnderestimation(const std::shared_ptr<base::State> q,
                                                 const std::shared_ptr<std::vector<Eigen::MatrixXf>> nearest_points) = 0;
};

}  // namespace base
