// Object.h -- RPMPLv2's env::Object (include/environments/Object.h:17-52)
// with the members the collision path reads: label, the fcl collision object
// (its world AABB), position, maximal velocity and min_dist_tol.
// setPosition moves the collision object and recomputes its AABB, as
// src/environments/Object.cpp:21-26 does.
#pragma once
#include <memory>
#include <string>

#include <fcl/fcl.h>

namespace env {

class Object {
public:
    Object() {}
    virtual ~Object() = 0;

    inline const std::string &getLabel() const { return label; }
    inline std::shared_ptr<fcl::CollisionObject<float>> getCollObject() const { return coll_object; }
    inline const fcl::Vector3f &getPosition() const { return position; }
    inline float getMaxVel() const { return max_vel; }
    inline float getMinDistTol() const { return min_dist_tol; }

    inline void setLabel(const std::string &label_) { label = label_; }
    void setPosition(const fcl::Vector3f &position_) {
        position = position_;
        coll_object->setTranslation(position);
        coll_object->computeAABB();
    }
    inline void setMaxVel(float max_vel_) { max_vel = max_vel_; }
    inline void setMinDistTol(float min_dist_tol_) { min_dist_tol = min_dist_tol_; }

protected:
    std::string label;
    std::shared_ptr<fcl::CollisionObject<float>> coll_object;
    fcl::Vector3f position;
    float max_vel = 0.f;
    float min_dist_tol = 1000.f;   // RealVectorSpaceConfig::MAX_DISTANCE
};

inline Object::~Object() {}

}  // namespace env
