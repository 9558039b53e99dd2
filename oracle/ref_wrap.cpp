// ref_wrap.cpp -- TEST INFRASTRUCTURE ONLY.
// C entry points around the reference's own static primitives
// (src/state_spaces/real_vector_space/CollisionAndDistance.cpp), compiled in
// place from the reference tree against the Eigen stand-in in
// oracle/eigen_standin.  Used only to pin the oracle's restatement.
#include "CollisionAndDistance.h"
#include "RealVectorSpaceConfig.h"

extern "C" {

void ref_set_config(float equality_threshold, float max_distance) {
    RealVectorSpaceConfig::EQUALITY_THRESHOLD = equality_threshold;
    RealVectorSpaceConfig::MAX_DISTANCE = max_distance;
}

int ref_collision(const float *A, const float *B, float r, const float *obs) {
    Eigen::Vector3f a(A[0], A[1], A[2]), b(B[0], B[1], B[2]);
    Eigen::VectorXf o(6);
    for (int k = 0; k < 6; ++k) o(k) = obs[k];
    return base::CollisionAndDistance::collisionCapsuleToBox(a, b, r, o) ? 1 : 0;
}

float ref_distance(const float *A, const float *B, float r, const float *obs, float *pts_out, int *has_pts) {
    Eigen::Vector3f a(A[0], A[1], A[2]), b(B[0], B[1], B[2]);
    Eigen::VectorXf o(6);
    for (int k = 0; k < 6; ++k) o(k) = obs[k];
    auto res = base::CollisionAndDistance::distanceCapsuleToBox(a, b, r, o);
    auto pts = std::get<1>(res);
    if (has_pts) *has_pts = pts ? 1 : 0;
    if (pts && pts_out)
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 3; ++i) pts_out[3 * j + i] = (*pts)(i, j);
    return std::get<0>(res);
}

float ref_segseg(const float *A, const float *B, const float *C, const float *D) {
    Eigen::Vector3f a(A[0], A[1], A[2]), b(B[0], B[1], B[2]), c(C[0], C[1], C[2]), d(D[0], D[1], D[2]);
    return std::get<0>(base::CollisionAndDistance::distanceLineSegToLineSeg(a, b, c, d));
}

}
