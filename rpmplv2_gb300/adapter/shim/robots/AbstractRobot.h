// AbstractRobot.h -- the accessors of RPMPLv2's robots::AbstractRobot
// (include/robots/AbstractRobot.h:21-82) that the collision and distance path
// reads, with the same names and members: type, DOFs, limits, capsule radii,
// gripper length and the ground rule.  Forward kinematics, IK and the mesh
// links are not part of the shim (the engine computes the skeleton itself).
#pragma once
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace robots {

class AbstractRobot {
public:
    explicit AbstractRobot() {}
    virtual ~AbstractRobot() = 0;

    inline const std::string &getType() const { return type; }
    inline size_t getNumDOFs() const { return num_DOFs; }
    inline const std::vector<std::pair<float, float>> &getLimits() const { return limits; }
    inline float getCapsuleRadius(size_t idx) const { return capsules_radius[idx]; }
    inline float getGripperLength() const { return gripper_length; }
    inline size_t getGroundIncluded() const { return ground_included; }
    inline bool getSelfCollisionChecking() const { return self_collision_checking; }

    inline virtual void setCapsulesRadius(const std::vector<float> &capsules_radius_) { capsules_radius = capsules_radius_; }
    inline void setGripperLength(float gripper_length_) { gripper_length = gripper_length_; }
    inline void setGroundIncluded(size_t ground_included_) { ground_included = ground_included_; }
    inline void setSelfCollisionChecking(bool self_collision_checking_) { self_collision_checking = self_collision_checking_; }

protected:
    std::string type;
    size_t num_DOFs = 0;
    std::vector<std::pair<float, float>> limits;
    std::vector<float> capsules_radius;
    bool self_collision_checking = false;
    float gripper_length = 0.f;
    size_t ground_included = 0;
};

inline AbstractRobot::~AbstractRobot() {}

}  // namespace robots
