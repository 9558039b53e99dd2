// RealVectorSpaceGPU.h -- base::RealVectorSpace on the GB300 engine.
//
// The four collision / distance virtuals of base::StateSpace are answered by
// the C ABI (include/rpm_gpu.h) with the reference's semantics, caches and
// write-backs (src/state_spaces/real_vector_space/RealVectorSpace.cpp):
//   isValid(q)                  :277-309, RPM_PREC_* arithmetic form of the space
//   isValid(q1, q2)             :261-275, NUM_INTERPOLATION_VALIDITY_CHECKS checks, q2 first
//   computeDistance(q, again)   :318-392, cached on q unless 'again'; writes d_c,
//                               its profile, is_real = true, the nearest points
//                               (nullptr after a collision) and the skeleton
//   computeDistanceUnderestimation(q, nearest) :402-446, cached on q; writes d_c,
//                               its profile and is_real = false unless it returns 0
// plus batched entry points for planners that check many states at once.
// The planners (RRTConnect, RGBTConnect, RGBMT*, DRGBT, RRTx) keep calling
// the virtuals and need no change.  The space owns one engine context, one
// robot, one device-resident scene and a small set of device staging buffers,
// and runs every call on its own stream.
//
// Built with the reference's constructor (robot and environment), the space
// keeps StateSpace::robot and StateSpace::env set, as planners expect
// (DRGBT.cpp:15, 31; MotionValidity.cpp:12-15), and follows the environment:
// before every check it compares each object's fcl world AABB with the device
// scene and sends what moved as one incremental update, so a planner that
// moves obstacles in place (env->updateEnvironment(dt) before ss->isValid(q),
// MotionValidity.cpp:39-42) is checked against the moved scene.  Objects added
// or removed, or a label or min_dist_tol changed, rebuild the scene.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include <environments/Environment.h>
#include <robots/AbstractRobot.h>
#include <state_spaces/real_vector_space/RealVectorSpace.h>

#include "rpm_gpu.h"

namespace base {

class RealVectorSpaceGPU : public RealVectorSpace {
public:
    // Obstacles as fcl world AABBs (n x 6: xmin ymin zmin xmax ymax zmax),
    // their min_dist_tol and RPM_OBS_* flags (label "ground" / "dynamic_obstacle").
    struct Obstacles {
        std::vector<float> aabb;
        std::vector<float> min_dist_tol;
        std::vector<uint8_t> flags;
    };

    // The reference's constructor (RealVectorSpace.h:21-22): the robot is
    // described by its type's URDF table (rpm_robot_builtin) with its own
    // capsule radii, ground rule and gripper length; the obstacles are the
    // environment's objects as RealVectorSpace.cpp:285-295 reads them (fcl
    // world AABB, label "ground" / "dynamic_obstacle", min_dist_tol).
    // 'precision' is an RPM_PREC_* form for the checks.
    RealVectorSpaceGPU(size_t num_dimensions, const std::shared_ptr<robots::AbstractRobot> robot,
                       const std::shared_ptr<env::Environment> env, int32_t precision = RPM_PREC_FP32_RECHECK,
                       int device = 0, int32_t num_interpolation_validity_checks = 10);
    // Without robot and environment objects: 'robot' is the kinematic table
    // the reference's robot builds from its URDF (rpm_robot_desc), and the
    // obstacles change only through updateObstacles.
    RealVectorSpaceGPU(const rpm_robot_desc &robot, const Obstacles &obstacles,
                       int32_t precision = RPM_PREC_FP32_RECHECK, int device = 0,
                       int32_t num_interpolation_validity_checks = 10);
    ~RealVectorSpaceGPU() override;
    RealVectorSpaceGPU(const RealVectorSpaceGPU &) = delete;
    RealVectorSpaceGPU &operator=(const RealVectorSpaceGPU &) = delete;

    bool isValid(const std::shared_ptr<base::State> q1, const std::shared_ptr<base::State> q2) override;
    bool isValid(const std::shared_ptr<base::State> q) override;
    float computeDistance(const std::shared_ptr<base::State> q, bool compute_again = false) override;
    float computeDistanceUnderestimation(const std::shared_ptr<base::State> q,
                                         const std::shared_ptr<std::vector<Eigen::MatrixXf>> nearest_points) override;

    // Batched forms: one launch for all states.  computeDistanceBatch writes
    // d_c, its profile and is_real = true on every state (no nearest points).
    std::vector<bool> isValidBatch(const std::vector<std::shared_ptr<base::State>> &qs);
    std::vector<float> computeDistanceBatch(const std::vector<std::shared_ptr<base::State>> &qs);
    std::vector<bool> isValidEdgesBatch(const std::vector<std::shared_ptr<base::State>> &q1s,
                                        const std::vector<std::shared_ptr<base::State>> &q2s);

    // Environment::updateEnvironment for moving obstacles: new AABBs of the
    // obstacles 'idx' (m x 6); returns the scene's new version.
    uint64_t updateObstacles(const std::vector<int32_t> &idx, const std::vector<float> &aabb);

    // Bring the device scene up to date with 'env' (every check does this
    // first); returns the scene's version.  No-op without an environment.
    uint64_t syncEnvironment();

    // The descriptor and obstacle arrays the constructor derives from the
    // reference's robot and environment objects.
    static rpm_robot_desc describe(const robots::AbstractRobot &robot);
    static Obstacles obstaclesOf(const env::Environment &env);

    inline rpm_ctx *context() const { return ctx_; }
    inline int32_t sceneId() const { return scene_; }

private:
    void init(const rpm_robot_desc &robot, const Obstacles &obstacles, int device);
    void createScene(const Obstacles &obstacles);
    void reserve(size_t configs);
    void upload(const std::vector<std::shared_ptr<base::State>> &qs, float *dst);
    void check(int rc) const;   // throws std::runtime_error with rpm_last_error_string()

    rpm_ctx *ctx_ = nullptr;
    int32_t robot_ = -1, scene_ = -1, prec_ = RPM_PREC_FP32_RECHECK, checks_ = 10;
    int D_ = 0, n_ = 0;
    Obstacles scene_obs_;       // what the device scene holds (syncEnvironment compares against it)
    uint64_t version_ = 0;
    void *stream_ = nullptr;
    size_t cap_ = 0;
    float *dq_ = nullptr, *dq2_ = nullptr, *dprof_ = nullptr, *dnear_ = nullptr;
    double *ddist_ = nullptr, *dskel_ = nullptr;
    uint8_t *dvalid_ = nullptr, *dflag_ = nullptr;
};

}  // namespace base
