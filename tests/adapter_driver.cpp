// adapter_driver.cpp -- TEST INFRASTRUCTURE: drives base::RealVectorSpaceGPU
// the way a planner does (shared_ptr states, the four virtuals, the batched
// forms) on inputs written by tests/test_gpu_adapter.py, and writes every
// output for the test to compare with the oracle.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "RealVectorSpaceGPU.h"

template <typename T> static void rd(FILE *f, T *p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input");
}
template <typename T> static void wr(FILE *f, const T *p, size_t n) {
    if (n) fwrite(p, sizeof(T), n, f);
}

static std::shared_ptr<base::State> state_of(const float *x, int D) {
    Eigen::VectorXf v(D);
    for (int k = 0; k < D; ++k) v(k) = x[k];
    return std::make_shared<base::RealVectorSpaceState>(v);
}

int main(int argc, char **argv) {
    if (argc != 3) { fprintf(stderr, "usage: adapter_driver in out\n"); return 2; }
    FILE *in = fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t hdr[5];
    rd(in, hdr, 5);
    const int prec = hdr[0], C = hdr[1], E = hdr[2], n = hdr[3], D = hdr[4];
    rpm_robot_desc desc;
    rd(in, reinterpret_cast<unsigned char *>(&desc), sizeof desc);
    base::RealVectorSpaceGPU::Obstacles ob;
    ob.aabb.resize((size_t)n * 6); ob.min_dist_tol.resize(n); ob.flags.resize(n);
    rd(in, ob.aabb.data(), ob.aabb.size()); rd(in, ob.min_dist_tol.data(), n); rd(in, ob.flags.data(), n);
    std::vector<float> q((size_t)C * D), q1((size_t)E * D), q2((size_t)E * D);
    rd(in, q.data(), q.size()); rd(in, q1.data(), q1.size()); rd(in, q2.data(), q2.size());
    fclose(in);

    base::RealVectorSpaceGPU space(desc, ob, prec);
    base::StateSpace &ss = space;   // planners hold the base interface
    const size_t NS = (size_t)n * 6 * D;
    std::vector<uint8_t> valid(C), valid_b(C), has_near(C), cached_ok(C), under_set(C), edge(E), edge_b(E);
    std::vector<float> dist(C), prof((size_t)C * D), near((size_t)C * NS, 0.f), skel((size_t)C * 3 * (D + 1));
    std::vector<float> under(C, NAN), under_prof((size_t)C * D, 0.f), dist_b(C);
    std::vector<std::shared_ptr<base::State>> states;
    for (int c = 0; c < C; ++c) states.push_back(state_of(&q[(size_t)c * D], D));
    for (int c = 0; c < C; ++c) {
        valid[c] = ss.isValid(states[c]) ? 1 : 0;
        dist[c] = ss.computeDistance(states[c]);
        const std::vector<float> &p = states[c]->getDistanceProfile();
        for (int i = 0; i < D; ++i) prof[(size_t)c * D + i] = p[i];
        auto np = states[c]->getNearestPoints();
        has_near[c] = np ? 1 : 0;
        if (np)
            for (int j = 0; j < n; ++j)
                for (int k = 0; k < 6; ++k)
                    for (int i = 0; i < D; ++i) near[(size_t)c * NS + ((size_t)j * 6 + k) * D + i] = (*np)[j](k, i);
        auto sk = states[c]->getSkeleton();
        for (int pnt = 0; pnt <= D; ++pnt)
            for (int k = 0; k < 3; ++k) skel[(size_t)c * 3 * (D + 1) + 3 * pnt + k] = (*sk)(k, pnt);
        // a second call answers from the state's cache (a real distance > 0), a forced one recomputes
        const float again = ss.computeDistance(states[c]);
        const float forced = ss.computeDistance(states[c], true);
        cached_ok[c] = (std::memcmp(&again, &dist[c], 4) == 0 && std::memcmp(&forced, &dist[c], 4) == 0) ? 1 : 0;
    }
    for (int c = 0; c < C; ++c) {
        // underestimation at the next configuration from this one's nearest points
        auto np = states[c]->getNearestPoints();
        if (!np) continue;
        auto p = state_of(&q[(size_t)((c + 1) % C) * D], D);
        under[c] = ss.computeDistanceUnderestimation(p, np);
        under_set[c] = (p->getDistance() != -1.f && !p->getIsRealDistance()) ? 1 : 0;
        if (under_set[c])
            for (int i = 0; i < D; ++i) under_prof[(size_t)c * D + i] = p->getDistanceProfile()[i];
    }
    std::vector<bool> vb = space.isValidBatch(states);
    for (int c = 0; c < C; ++c) valid_b[c] = vb[c] ? 1 : 0;
    std::vector<std::shared_ptr<base::State>> fresh;
    for (int c = 0; c < C; ++c) fresh.push_back(state_of(&q[(size_t)c * D], D));
    std::vector<float> db = space.computeDistanceBatch(fresh);
    for (int c = 0; c < C; ++c) dist_b[c] = db[c];
    std::vector<std::shared_ptr<base::State>> s1, s2;
    for (int e = 0; e < E; ++e) {
        s1.push_back(state_of(&q1[(size_t)e * D], D));
        s2.push_back(state_of(&q2[(size_t)e * D], D));
        edge[e] = ss.isValid(s1.back(), s2.back()) ? 1 : 0;
    }
    std::vector<bool> eb = space.isValidEdgesBatch(s1, s2);
    for (int e = 0; e < E; ++e) edge_b[e] = eb[e] ? 1 : 0;

    FILE *out = fopen(argv[2], "wb");
    if (!out) return 2;
    wr(out, valid.data(), C); wr(out, valid_b.data(), C); wr(out, dist.data(), C); wr(out, prof.data(), prof.size());
    wr(out, has_near.data(), C); wr(out, near.data(), near.size()); wr(out, cached_ok.data(), C);
    wr(out, skel.data(), skel.size()); wr(out, under.data(), C); wr(out, under_set.data(), C);
    wr(out, under_prof.data(), under_prof.size()); wr(out, dist_b.data(), C); wr(out, edge.data(), E);
    wr(out, edge_b.data(), E);
    fclose(out);
    return 0;
}
