// Box.h -- RPMPLv2's env::Box (include/environments/Box.h, built as in
// src/environments/objects/Box.cpp:3-14): an fcl box at 'pos' with rotation
// 'rot', its AABB computed at construction, min_dist_tol = MAX_DISTANCE.
#pragma once
#include "Object.h"

namespace env {

class Box : public Object {
public:
    Box(const fcl::Vector3f &dim, const fcl::Vector3f &pos, const fcl::Quaternionf &rot, const std::string &label_ = "") {
        coll_object = std::make_shared<fcl::CollisionObject<float>>(dim, rot, pos);
        coll_object->computeAABB();
        position = pos;
        label = label_;
    }
    ~Box() {}
};

}  // namespace env
