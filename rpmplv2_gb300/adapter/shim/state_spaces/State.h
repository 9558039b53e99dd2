// State.h -- the part of RPMPLv2's base::State (include/state_spaces/State.h)
// that the collision and distance path reads and writes, with the same names
// and signatures: coordinates, the distance-to-obstacles d_c and its per-link
// profile, whether d_c is real or an underestimation, the nearest points and
// the skeleton.  A new state starts with d_c = -1 (src/state_spaces/State.cpp).
#pragma once
#include <eigen3/Eigen/Dense>
#include <memory>
#include <vector>

namespace base {

class State {
public:
    enum class Status { None, Advanced, Trapped, Reached, Orphan };

protected:
    size_t num_dimensions;
    Eigen::VectorXf coord;
    float d_c;
    std::vector<float> d_c_profile;
    bool is_real_d_c;
    std::shared_ptr<std::vector<Eigen::MatrixXf>> nearest_points;
    std::shared_ptr<Eigen::MatrixXf> skeleton;
    Status status;

public:
    State(const Eigen::VectorXf &coord_)
        : num_dimensions((size_t)coord_.size()), coord(coord_), d_c(-1), is_real_d_c(true), status(Status::None) {}
    virtual ~State() = 0;

    inline size_t getNumDimensions() const { return num_dimensions; }
    inline const Eigen::VectorXf &getCoord() const { return coord; }
    inline float getCoord(size_t idx) const { return coord((Eigen::Index)idx); }
    inline float getDistance() const { return d_c; }
    inline const std::vector<float> &getDistanceProfile() const { return d_c_profile; }
    inline float getDistanceProfile(size_t idx) { return d_c_profile[idx]; }
    inline bool getIsRealDistance() const { return is_real_d_c; }
    inline std::shared_ptr<std::vector<Eigen::MatrixXf>> getNearestPoints() const { return nearest_points; }
    inline std::shared_ptr<Eigen::MatrixXf> getSkeleton() const { return skeleton; }
    inline Status getStatus() const { return status; }

    inline void setCoord(const Eigen::VectorXf &coord_) { coord = coord_; }
    inline void setDistance(float d_c_) { d_c = d_c_; }
    inline void setDistanceProfile(const std::vector<float> &d_c_profile_) { d_c_profile = d_c_profile_; }
    inline void setIsRealDistance(bool is_real_d_c_) { is_real_d_c = is_real_d_c_; }
    inline void setNearestPoints(const std::shared_ptr<std::vector<Eigen::MatrixXf>> nearest_points_) {
        nearest_points = nearest_points_;
    }
    inline void setSkeleton(const std::shared_ptr<Eigen::MatrixXf> skeleton_) { skeleton = skeleton_; }
    inline void setStatus(Status status_) { status = status_; }
};

inline State::~State() {}

}  // namespace base
