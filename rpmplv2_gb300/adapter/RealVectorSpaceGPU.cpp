// RealVectorSpaceGPU.cpp -- see RealVectorSpaceGPU.h.
#include "RealVectorSpaceGPU.h"

#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>

namespace base {

namespace {
void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace

void RealVectorSpaceGPU::check(int rc) const {
    if (rc != RPM_OK) throw std::runtime_error(std::string("rpm: ") + rpm_last_error_string());
}

rpm_robot_desc RealVectorSpaceGPU::describe(const robots::AbstractRobot &robot) {
    rpm_robot_desc d;
    if (rpm_robot_builtin(robot.getType().c_str(), &d) != RPM_OK)
        throw std::invalid_argument(std::string("RealVectorSpaceGPU: ") + rpm_last_error_string());
    if (robot.getNumDOFs() != (size_t)d.num_dofs)
        throw std::invalid_argument("RealVectorSpaceGPU: the robot's DOF count differs from its type's URDF");
    for (int i = 0; i < d.num_dofs; ++i) d.capsule_radius[i] = robot.getCapsuleRadius((size_t)i);
    d.ground_included = (int32_t)robot.getGroundIncluded();
    d.gripper_length = robot.getGripperLength();
    const auto &lim = robot.getLimits();
    for (int i = 0; i < d.num_dofs && i < (int)lim.size(); ++i) {
        d.limits[i][0] = lim[i].first;
        d.limits[i][1] = lim[i].second;
    }
    return d;
}

// The objects as RealVectorSpace.cpp:285-295 and :344-346 read them: the fcl
// world AABB (min_, max_), the "ground" label for the ground rule, the
// "dynamic_obstacle" label for moving boxes, and Object::getMinDistTol.
RealVectorSpaceGPU::Obstacles RealVectorSpaceGPU::obstaclesOf(const env::Environment &env) {
    Obstacles o;
    const size_t n = env.getNumObjects();
    o.aabb.resize(6 * n);
    o.min_dist_tol.resize(n);
    o.flags.resize(n);
    for (size_t j = 0; j < n; ++j) {
        const auto &box = env.getCollObject(j)->getAABB();
        for (int k = 0; k < 3; ++k) {
            o.aabb[6 * j + k] = box.min_[k];
            o.aabb[6 * j + 3 + k] = box.max_[k];
        }
        const std::string &label = env.getObject(j)->getLabel();
        o.min_dist_tol[j] = env.getObject(j)->getMinDistTol();
        o.flags[j] = (uint8_t)((label == "ground" ? RPM_OBS_GROUND : 0u) | (label == "dynamic_obstacle" ? RPM_OBS_DYNAMIC : 0u));
    }
    return o;
}

RealVectorSpaceGPU::RealVectorSpaceGPU(size_t num_dimensions, const std::shared_ptr<robots::AbstractRobot> robot,
                                       const std::shared_ptr<env::Environment> env, int32_t precision, int device,
                                       int32_t num_interpolation_validity_checks)
    : RealVectorSpace(num_dimensions, robot, env), prec_(precision), checks_(num_interpolation_validity_checks) {
    if (!robot || !env) throw std::invalid_argument("RealVectorSpaceGPU: robot and environment are required");
    const rpm_robot_desc desc = describe(*robot);
    if ((size_t)desc.num_dofs != num_dimensions)
        throw std::invalid_argument("RealVectorSpaceGPU: num_dimensions differs from the robot's DOF count");
    init(desc, obstaclesOf(*env), device);
}

RealVectorSpaceGPU::RealVectorSpaceGPU(const rpm_robot_desc &robot, const Obstacles &obstacles, int32_t precision,
                                       int device, int32_t num_interpolation_validity_checks)
    : RealVectorSpace((size_t)robot.num_dofs), prec_(precision), checks_(num_interpolation_validity_checks) {
    init(robot, obstacles, device);
}

void RealVectorSpaceGPU::init(const rpm_robot_desc &robot, const Obstacles &obstacles, int device) {
    check(rpm_ctx_create(device, &ctx_));
    check(rpm_robot_upload(ctx_, &robot, &robot_));
    D_ = robot.num_dofs;
    createScene(obstacles);
    cudaStream_t st;
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    stream_ = st;
    reserve(1);
}

void RealVectorSpaceGPU::createScene(const Obstacles &obstacles) {
    const int n = (int)(obstacles.aabb.size() / 6);
    if (obstacles.aabb.size() != 6 * (size_t)n || (!obstacles.min_dist_tol.empty() && obstacles.min_dist_tol.size() != (size_t)n) ||
        (!obstacles.flags.empty() && obstacles.flags.size() != (size_t)n))
        throw std::invalid_argument("RealVectorSpaceGPU: obstacle arrays of inconsistent sizes");
    if (scene_ >= 0) {
        check(rpm_sync(ctx_, stream_));   // checks still reading the old scene finish first
        check(rpm_scene_destroy(ctx_, scene_));
        scene_ = -1;
    }
    check(rpm_scene_create(ctx_, robot_, n ? obstacles.aabb.data() : nullptr,
                           obstacles.min_dist_tol.empty() ? nullptr : obstacles.min_dist_tol.data(),
                           obstacles.flags.empty() ? nullptr : obstacles.flags.data(), n, &scene_));
    check(rpm_scene_info(ctx_, scene_, nullptr, nullptr, &version_));
    const bool grew = n > n_;
    n_ = n;
    scene_obs_ = obstacles;
    if (grew && cap_ > 0) {   // the nearest-point buffer is sized by the obstacle count
        const size_t c = cap_;
        cap_ = 0;
        reserve(c);
    }
}

uint64_t RealVectorSpaceGPU::syncEnvironment() {
    if (!env) return version_;
    const Obstacles cur = obstaclesOf(*env);
    const size_t n = cur.min_dist_tol.size();
    if (n != (size_t)n_ || cur.min_dist_tol != scene_obs_.min_dist_tol || cur.flags != scene_obs_.flags) {
        createScene(cur);
        return version_;
    }
    std::vector<int32_t> idx;
    std::vector<float> rows;
    for (size_t j = 0; j < n; ++j) {
        if (std::memcmp(&cur.aabb[6 * j], &scene_obs_.aabb[6 * j], 6 * sizeof(float)) == 0) continue;
        idx.push_back((int32_t)j);
        rows.insert(rows.end(), cur.aabb.begin() + 6 * j, cur.aabb.begin() + 6 * (j + 1));
    }
    if (!idx.empty()) {
        check(rpm_scene_update(ctx_, scene_, idx.data(), rows.data(), (int32_t)idx.size(), &version_));
        scene_obs_.aabb = cur.aabb;
    }
    return version_;
}

RealVectorSpaceGPU::~RealVectorSpaceGPU() {
    cudaFree(dq_); cudaFree(dq2_); cudaFree(dprof_); cudaFree(dnear_); cudaFree(ddist_); cudaFree(dskel_);
    cudaFree(dvalid_); cudaFree(dflag_);
    if (stream_) cudaStreamDestroy((cudaStream_t)stream_);
    if (ctx_) rpm_ctx_destroy(ctx_);
}

void RealVectorSpaceGPU::reserve(size_t configs) {
    if (configs <= cap_) return;
    cudaFree(dq_); cudaFree(dq2_); cudaFree(dprof_); cudaFree(dnear_); cudaFree(ddist_); cudaFree(dskel_);
    cudaFree(dvalid_); cudaFree(dflag_);
    const size_t c = configs;
    cuda_check(cudaMalloc(&dq_, c * D_ * sizeof(float)), "cudaMalloc");
    cuda_check(cudaMalloc(&dq2_, c * D_ * sizeof(float)), "cudaMalloc");
    cuda_check(cudaMalloc(&dprof_, c * D_ * sizeof(float)), "cudaMalloc");
    cuda_check(cudaMalloc(&ddist_, c * sizeof(double)), "cudaMalloc");
    cuda_check(cudaMalloc(&dskel_, 3 * (D_ + 1) * sizeof(double)), "cudaMalloc");
    cuda_check(cudaMalloc(&dvalid_, c), "cudaMalloc");
    cuda_check(cudaMalloc(&dflag_, c), "cudaMalloc");
    cuda_check(cudaMalloc(&dnear_, (size_t)(n_ ? n_ : 1) * 6 * D_ * sizeof(float)), "cudaMalloc");
    cap_ = c;
}

void RealVectorSpaceGPU::upload(const std::vector<std::shared_ptr<base::State>> &qs, float *dst) {
    std::vector<float> h(qs.size() * D_);
    for (size_t c = 0; c < qs.size(); ++c) {
        const Eigen::VectorXf &x = qs[c]->getCoord();
        if (x.size() != D_) throw std::invalid_argument("RealVectorSpaceGPU: state of the wrong dimension");
        for (int k = 0; k < D_; ++k) h[c * D_ + k] = x(k);
    }
    cuda_check(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, (cudaStream_t)stream_),
               "cudaMemcpyAsync");
}

bool RealVectorSpaceGPU::isValid(const std::shared_ptr<base::State> q) { return isValidBatch({q})[0]; }

bool RealVectorSpaceGPU::isValid(const std::shared_ptr<base::State> q1, const std::shared_ptr<base::State> q2) {
    return isValidEdgesBatch({q1}, {q2})[0];
}

// computeDistance (RealVectorSpace.cpp:318-392): the cached value when it is a
// real distance and 'compute_again' is not set; otherwise every pair with
// nearest points, written back to the state.  The nearest points come from an
// exact form (the reference's FP32 numerics for RPM_PREC_FP32_REF, FP64
// otherwise).
float RealVectorSpaceGPU::computeDistance(const std::shared_ptr<base::State> q, bool compute_again) {
    if (!compute_again && q->getDistance() > 0 && q->getIsRealDistance()) return q->getDistance();
    syncEnvironment();
    upload({q}, dq_);
    cudaStream_t st = (cudaStream_t)stream_;
    const int32_t form = prec_ == RPM_PREC_FP32_REF ? RPM_PREC_FP32_REF : RPM_PREC_FP64;
    check(rpm_distance_nearest(ctx_, scene_, form, dq_, 1, ddist_, dprof_, dnear_, dflag_, stream_));
    check(rpm_skeleton(ctx_, robot_, RPM_PREC_FP32_REF, dq_, 1, dskel_, stream_));
    double d = 0;
    uint8_t valid = 0;
    std::vector<float> prof(D_);
    std::vector<float> near((size_t)n_ * 6 * D_);
    std::vector<double> skel(3 * (D_ + 1));
    cuda_check(cudaMemcpyAsync(&d, ddist_, sizeof d, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    cuda_check(cudaMemcpyAsync(&valid, dflag_, 1, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    cuda_check(cudaMemcpyAsync(prof.data(), dprof_, prof.size() * sizeof(float), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync");
    if (!near.empty())
        cuda_check(cudaMemcpyAsync(near.data(), dnear_, near.size() * sizeof(float), cudaMemcpyDeviceToHost, st),
                   "cudaMemcpyAsync");
    cuda_check(cudaMemcpyAsync(skel.data(), dskel_, skel.size() * sizeof(double), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    auto sk = std::make_shared<Eigen::MatrixXf>(3, D_ + 1);
    for (int p = 0; p <= D_; ++p)
        for (int k = 0; k < 3; ++k) (*sk)(k, p) = (float)skel[3 * p + k];
    q->setSkeleton(sk);
    q->setDistance((float)d);
    q->setDistanceProfile(prof);
    q->setIsRealDistance(true);
    if (valid) {
        auto np = std::make_shared<std::vector<Eigen::MatrixXf>>((size_t)n_, Eigen::MatrixXf(6, D_));
        for (int j = 0; j < n_; ++j)
            for (int k = 0; k < 6; ++k)
                for (int i = 0; i < D_; ++i) (*np)[j](k, i) = near[((size_t)j * 6 + k) * D_ + i];
        q->setNearestPoints(np);
    } else {
        q->setNearestPoints(nullptr);
    }
    return (float)d;
}

// computeDistanceUnderestimation (RealVectorSpace.cpp:402-446).
float RealVectorSpaceGPU::computeDistanceUnderestimation(const std::shared_ptr<base::State> q,
                                                         const std::shared_ptr<std::vector<Eigen::MatrixXf>> nearest_points) {
    if (q->getDistance() > 0 && q->getIsRealDistance()) return q->getDistance();
    if (!nearest_points || nearest_points->size() != (size_t)n_)
        throw std::invalid_argument("RealVectorSpaceGPU: nearest points of another environment");
    std::vector<float> near((size_t)n_ * 6 * D_);
    for (int j = 0; j < n_; ++j) {
        const Eigen::MatrixXf &m = (*nearest_points)[j];
        if (m.rows() != 6 || m.cols() != D_) throw std::invalid_argument("RealVectorSpaceGPU: nearest points of another robot");
        for (int k = 0; k < 6; ++k)
            for (int i = 0; i < D_; ++i) near[((size_t)j * 6 + k) * D_ + i] = m(k, i);
    }
    syncEnvironment();
    cudaStream_t st = (cudaStream_t)stream_;
    upload({q}, dq_);
    if (!near.empty())
        cuda_check(cudaMemcpyAsync(dnear_, near.data(), near.size() * sizeof(float), cudaMemcpyHostToDevice, st),
                   "cudaMemcpyAsync");
    const int32_t form = prec_ == RPM_PREC_FP32_REF ? RPM_PREC_FP32_REF : RPM_PREC_FP64;
    check(rpm_distance_underestimation(ctx_, scene_, form, dq_, 1, dnear_, ddist_, dprof_, dflag_, stream_));
    double d = 0;
    uint8_t complete = 0;
    std::vector<float> prof(D_);
    cuda_check(cudaMemcpyAsync(&d, ddist_, sizeof d, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    cuda_check(cudaMemcpyAsync(&complete, dflag_, 1, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    cuda_check(cudaMemcpyAsync(prof.data(), dprof_, prof.size() * sizeof(float), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (!complete) return 0;   // the reference returns 0 without updating the state
    q->setDistance((float)d);
    q->setDistanceProfile(prof);
    q->setIsRealDistance(false);
    return (float)d;
}

std::vector<bool> RealVectorSpaceGPU::isValidBatch(const std::vector<std::shared_ptr<base::State>> &qs) {
    std::vector<bool> out(qs.size());
    if (qs.empty()) return out;
    syncEnvironment();
    reserve(qs.size());
    upload(qs, dq_);
    cudaStream_t st = (cudaStream_t)stream_;
    check(rpm_check_configs(ctx_, scene_, prec_, dq_, (int64_t)qs.size(), dvalid_, nullptr, nullptr, stream_));
    std::vector<uint8_t> v(qs.size());
    cuda_check(cudaMemcpyAsync(v.data(), dvalid_, v.size(), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    for (size_t c = 0; c < qs.size(); ++c) out[c] = v[c] != 0;
    return out;
}

std::vector<float> RealVectorSpaceGPU::computeDistanceBatch(const std::vector<std::shared_ptr<base::State>> &qs) {
    std::vector<float> out(qs.size());
    if (qs.empty()) return out;
    syncEnvironment();
    reserve(qs.size());
    upload(qs, dq_);
    cudaStream_t st = (cudaStream_t)stream_;
    check(rpm_check_configs(ctx_, scene_, prec_, dq_, (int64_t)qs.size(), nullptr, ddist_, dprof_, stream_));
    std::vector<double> d(qs.size());
    std::vector<float> prof(qs.size() * D_);
    cuda_check(cudaMemcpyAsync(d.data(), ddist_, d.size() * sizeof(double), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync");
    cuda_check(cudaMemcpyAsync(prof.data(), dprof_, prof.size() * sizeof(float), cudaMemcpyDeviceToHost, st),
               "cudaMemcpyAsync");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    for (size_t c = 0; c < qs.size(); ++c) {
        out[c] = (float)d[c];
        qs[c]->setDistance(out[c]);
        qs[c]->setDistanceProfile(std::vector<float>(prof.begin() + c * D_, prof.begin() + (c + 1) * D_));
        qs[c]->setIsRealDistance(true);
    }
    return out;
}

std::vector<bool> RealVectorSpaceGPU::isValidEdgesBatch(const std::vector<std::shared_ptr<base::State>> &q1s,
                                                        const std::vector<std::shared_ptr<base::State>> &q2s) {
    if (q1s.size() != q2s.size()) throw std::invalid_argument("RealVectorSpaceGPU: edge lists of different lengths");
    std::vector<bool> out(q1s.size());
    if (q1s.empty()) return out;
    syncEnvironment();
    reserve(q1s.size());
    upload(q1s, dq_);
    upload(q2s, dq2_);
    cudaStream_t st = (cudaStream_t)stream_;
    check(rpm_check_edges(ctx_, scene_, prec_, dq_, dq2_, (int64_t)q1s.size(), 0.f, checks_, dvalid_, nullptr, stream_));
    std::vector<uint8_t> v(q1s.size());
    cuda_check(cudaMemcpyAsync(v.data(), dvalid_, v.size(), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    for (size_t e = 0; e < q1s.size(); ++e) out[e] = v[e] != 0;
    return out;
}

uint64_t RealVectorSpaceGPU::updateObstacles(const std::vector<int32_t> &idx, const std::vector<float> &aabb) {
    if (aabb.size() != 6 * idx.size()) throw std::invalid_argument("RealVectorSpaceGPU: 6 AABB values per obstacle");
    for (int32_t j : idx)
        if (j < 0 || j >= n_) throw std::invalid_argument("RealVectorSpaceGPU: obstacle index out of range");
    check(rpm_scene_update(ctx_, scene_, idx.data(), aabb.data(), (int32_t)idx.size(), &version_));
    for (size_t k = 0; k < idx.size(); ++k)
        std::memcpy(&scene_obs_.aabb[6 * (size_t)idx[k]], &aabb[6 * k], 6 * sizeof(float));
    return version_;
}

}  // namespace base
