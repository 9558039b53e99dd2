// StateSpace.h -- the collision and distance interface of RPMPLv2's
// base::StateSpace (include/state_spaces/StateSpace.h:16-57), with the same
// signatures.  Planners call these four virtuals; nothing else of the state
// space is needed by the path.
#pragma once
#include <memory>
#include <vector>

#include "State.h"

namespace base {

class StateSpace {
public:
    size_t num_dimensions;

    StateSpace(size_t num_dimensions_) : num_dimensions(num_dimensions_) {}
    virtual ~StateSpace() {}
    inline size_t getNumDimensions() { return num_dimensions; }

    virtual bool isValid(const std::shared_ptr<base::State> q) = 0;
    virtual bool isValid(const std::shared_ptr<base::State> q1, const std::shared_ptr<base::State> q2) = 0;
    virtual float computeDistance(const std::shared_ptr<base::State> q, bool compute_again = false) = 0;
    virtual float computeDistanceUnderestimation(const std::shared_ptr<base::State> q,
                                                 const std::shared_ptr<std::vector<Eigen::MatrixXf>> nearest_points) = 0;
};

}  // namespace base
