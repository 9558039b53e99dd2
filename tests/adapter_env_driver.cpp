// adapter_env_driver.cpp -- TEST INFRASTRUCTURE: base::RealVectorSpaceGPU built
// the reference's way, from a robots::AbstractRobot and an env::Environment
// (RealVectorSpace.h:21-22), then driven the way MotionValidity::check drives
// a state space (MotionValidity.cpp:30-53): the planner moves the obstacles
// in place with env->updateEnvironment(dt) and then calls ss->isValid(q) and
// ss->computeDistance(q) through the base interface.  Writes each step's
// obstacle AABBs (as the environment holds them) and every result, for
// tests/test_gpu_adapter.py to compare with the oracle on those AABBs.
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "RealVectorSpaceGPU.h"

template <typename T> static void rd(FILE *f, T *p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input");
}
template <typename T> static void wr(FILE *f, const T *p, size_t n) {
    if (n) fwrite(p, sizeof(T), n, f);
}

// A robot as the reference's scenario builds it: type, DOFs, limits, then
// setCapsulesRadius / setGroundIncluded / setGripperLength.
class DriverRobot : public robots::AbstractRobot {
public:
    DriverRobot(const std::string &type_, size_t dofs) {
        type = type_;
        num_DOFs = dofs;
        limits.assign(dofs, {-3.14159f, 3.14159f});
    }
};

static std::shared_ptr<base::State> state_of(const float *x, int D) {
    Eigen::VectorXf v(D);
    for (int k = 0; k < D; ++k) v(k) = x[k];
    return std::make_shared<base::RealVectorSpaceState>(v);
}

static void write_aabbs(FILE *out, const env::Environment &e) {
    for (size_t j = 0; j < e.getNumObjects(); ++j) {
        const auto &b = e.getCollObject(j)->getAABB();
        const float v[6] = {b.min_[0], b.min_[1], b.min_[2], b.max_[0], b.max_[1], b.max_[2]};
        wr(out, v, 6);
    }
}

int main(int argc, char **argv) {
    if (argc != 3) { fprintf(stderr, "usage: adapter_env_driver in out\n"); return 2; }
    FILE *in = fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t hdr[6];
    rd(in, hdr, 6);
    const int prec = hdr[0], S = hdr[1], K = hdr[2], n = hdr[3], D = hdr[4], ground = hdr[5];
    char type[32];
    rd(in, type, 32);
    type[31] = 0;
    std::vector<float> radii(D), boxes((size_t)n * 12), q((size_t)(S + 1) * K * D), extra(12);
    float gripper = 0.f, dt = 0.f;
    rd(in, radii.data(), D); rd(in, &gripper, 1); rd(in, &dt, 1);
    rd(in, boxes.data(), boxes.size()); rd(in, extra.data(), 12); rd(in, q.data(), q.size());
    fclose(in);

    auto robot = std::make_shared<DriverRobot>(type, (size_t)D);
    robot->setCapsulesRadius(radii);
    robot->setGroundIncluded((size_t)ground);
    robot->setGripperLength(gripper);
    // a box record: dim, pos, quat (x, y, z, w), label code (0 none, 1 "ground",
    // 2 "dynamic_obstacle"), then max_vel for a dynamic box or min_dist_tol
    // (0: MAX_DISTANCE) for the others
    auto make_box = [](const float *b) {
        const char *labels[3] = {"", "ground", "dynamic_obstacle"};
        const int code = (int)b[10];
        auto box = std::make_shared<env::Box>(fcl::Vector3f(b[0], b[1], b[2]), fcl::Vector3f(b[3], b[4], b[5]),
                                              fcl::Quaternionf(b[9], b[6], b[7], b[8]), labels[code]);
        if (code == 2) box->setMaxVel(b[11]);
        else if (b[11] > 0) box->setMinDistTol(b[11]);
        return box;
    };
    auto environment = std::make_shared<env::Environment>();
    for (int j = 0; j < n; ++j) environment->addObject(make_box(&boxes[(size_t)j * 12]));

    std::shared_ptr<base::StateSpace> ss =
        std::make_shared<base::RealVectorSpaceGPU>((size_t)D, robot, environment, prec);
    if (ss->robot != robot || ss->env != environment) { fprintf(stderr, "robot / env not kept\n"); return 3; }

    FILE *out = fopen(argv[2], "wb");
    if (!out) return 2;
    // step 0: the environment as built; steps 1..S: after env->updateEnvironment(dt);
    // step S+1: after removing object 0 and adding one more box (the scene is rebuilt)
    for (int s = 0; s <= S + 1; ++s) {
        if (s > 0 && s <= S) ss->env->updateEnvironment(dt);
        if (s == S + 1) {
            ss->env->removeObject(0);
            ss->env->addObject(make_box(extra.data()));
        }
        const int32_t cnt = (int32_t)ss->env->getNumObjects();
        wr(out, &cnt, 1);
        write_aabbs(out, *ss->env);
        const int row = s <= S ? s : S;
        for (int k = 0; k < K; ++k) {
            auto st = state_of(&q[((size_t)row * K + k) * D], D);
            const uint8_t v = ss->isValid(st) ? 1 : 0;
            const float d = ss->computeDistance(st, true);
            wr(out, &v, 1);
            wr(out, &d, 1);
        }
    }
    fclose(out);
    return 0;
}
