// fcl.h -- the part of fcl 0.7 that the RealVectorSpace path reads: a box
// collision object and its world AABB (getAABB().min_ / .max_, as
// RealVectorSpace.cpp:293-295 reads it), so the adapter builds where fcl is not
// installed.  Inside RPMPLv2 the adapter is compiled against the real fcl.
// The world AABB follows fcl's rule for a box, computed by the engine's
// rpm_box_aabb: identity rotation gives pos +- dim/2, any other rotation the
// cube pos +- |dim/2|.
#pragma once
#include <eigen3/Eigen/Dense>

#include "rpm_gpu.h"

namespace fcl {

typedef Eigen::Vector3f Vector3f;
typedef Eigen::Quaternionf Quaternionf;

template <typename S> struct AABB {
    Vector3f min_, max_;
};

template <typename S> class CollisionObject {
public:
    CollisionObject(const Vector3f &dim, const Quaternionf &rot, const Vector3f &pos)
        : dim_(dim), rot_(rot), pos_(pos) {}
    const AABB<S> &getAABB() const { return aabb_; }
    void setTranslation(const Vector3f &t) { pos_ = t; }
    const Vector3f &getTranslation() const { return pos_; }
    void computeAABB() {
        const float q[4] = {rot_.x(), rot_.y(), rot_.z(), rot_.w()};
        float out[6];
        rpm_box_aabb(dim_.data(), pos_.data(), q, out);
        aabb_.min_ = Vector3f(out[0], out[1], out[2]);
        aabb_.max_ = Vector3f(out[3], out[4], out[5]);
    }

private:
    Vector3f dim_;
    Quaternionf rot_;
    Vector3f pos_;
    AABB<S> aabb_;
};

typedef CollisionObject<float> CollisionObjectf;

}  // namespace fcl
