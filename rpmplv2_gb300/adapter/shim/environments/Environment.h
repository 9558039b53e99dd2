// Environment.h -- RPMPLv2's env::Environment (include/environments/Environment.h:17-80)
// as the collision path and its callers use it: the object list and its
// accessors (getObjects, getCollObject, getNumObjects), addObject /
// removeObject, and updateEnvironment with the straight-line motion law of
// Environment.cpp:220-233 (each "dynamic_obstacle" moves by -delta_time *
// max_vel along x, in float).  Planners mutate it in place; the adapter
// notices the change before its next check.  The YAML constructor and the
// other motion laws are not part of the shim.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "Box.h"

namespace env {

class Environment {
public:
    Environment() {}
    ~Environment() {}

    inline const std::vector<std::shared_ptr<env::Object>> &getObjects() const { return objects; }
    inline std::shared_ptr<env::Object> getObject(size_t idx) const { return objects[idx]; }
    inline std::shared_ptr<fcl::CollisionObjectf> getCollObject(size_t idx) const { return objects[idx]->getCollObject(); }
    inline size_t getNumObjects() const { return objects.size(); }

    void addObject(const std::shared_ptr<env::Object> object) { objects.emplace_back(object); }
    void removeObject(size_t idx) { objects.erase(objects.begin() + (long)idx); }

    void updateEnvironment(float delta_time) {
        for (size_t i = 0; i < objects.size(); i++) {
            if (objects[i]->getLabel() != "dynamic_obstacle") continue;
            fcl::Vector3f pos = objects[i]->getPosition();
            pos.x() -= delta_time * objects[i]->getMaxVel();
            objects[i]->setPosition(pos);
        }
    }

private:
    std::vector<std::shared_ptr<env::Object>> objects;
};

}  // namespace env
