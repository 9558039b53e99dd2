// rpm_io.cu -- scene I/O: the reference's scenario files into device-ready
// obstacle arrays (host code only).
//
//   rpm_scenario_read         a scenario YAML (data/<robot>/<scenario>/*.yaml) as
//                             Environment::Environment (Environment.cpp:13-109)
//                             and Scenario.cpp read it: box obstacles with
//                             label, dim, pos, optional rot [x, y, z, w] and
//                             min_dist_tol; the robot's type, DOFs, capsule
//                             radii, gripper length, ground_included,
//                             workspace and start / goal.
//   rpm_random_scenario_read  one run of random_scenarios.yaml
//                             (apps/test_drgbt_random_obstacles.cpp:125-151):
//                             start, goal and the objects' positions and
//                             velocities.
//   rpm_robot_builtin         the kinematic table of each of the reference's
//                             robots, by its type name (the URDF robot name).
//
// The files use a small part of YAML: block mappings and sequences by
// indentation, "- key: value" items, one-line flow sequences of scalars,
// quoted or plain scalars and # comments.  A reader of exactly that part is
// below (yaml-cpp, which the reference uses, is not available here).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "rpm_ctx_impl.cuh"

namespace rpm {
namespace impl {
namespace {

struct YNode {
    enum Kind { Null, Scalar, Seq, Map } kind = Null;
    std::string text;                                   // Scalar
    std::vector<std::shared_ptr<YNode>> items;          // Seq
    std::vector<std::pair<std::string, std::shared_ptr<YNode>>> fields;   // Map, in file order
    const YNode *get(const std::string &k) const {
        if (kind != Map) return nullptr;
        for (const auto &f : fields)
            if (f.first == k) return f.second.get();
        return nullptr;
    }
};
typedef std::shared_ptr<YNode> YPtr;

struct YLine {
    int indent;
    std::string text;   // without indentation and comment
};

std::string trim(const std::string &s) {
    size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// Strip a # comment that is not inside quotes.
std::string strip_comment(const std::string &s) {
    char q = 0;
    for (size_t i = 0; i < s.size(); ++i) {
        const char c = s[i];
        if (q) { if (c == q) q = 0; continue; }
        if (c == '"' || c == '\'') q = c;
        else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) return s.substr(0, i);
    }
    return s;
}

YPtr scalar(const std::string &raw) {
    auto n = std::make_shared<YNode>();
    std::string t = trim(raw);
    if (t.empty()) return n;   // null
    if (t.size() >= 2 && ((t.front() == '"' && t.back() == '"') || (t.front() == '\'' && t.back() == '\'')))
        t = t.substr(1, t.size() - 2);
    n->kind = YNode::Scalar;
    n->text = t;
    return n;
}

// A value on the same line as its key: a flow sequence or a scalar.
YPtr inline_value(const std::string &raw, bool &ok) {
    const std::string t = trim(raw);
    if (!t.empty() && t.front() == '[') {
        if (t.back() != ']') { ok = false; return nullptr; }
        auto n = std::make_shared<YNode>();
        n->kind = YNode::Seq;
        std::string body = t.substr(1, t.size() - 2), cur;
        std::stringstream ss(body);
        while (std::getline(ss, cur, ','))
            if (!trim(cur).empty()) n->items.push_back(scalar(cur));
        return n;
    }
    return scalar(t);
}

// "key: rest" -> key, rest (false if the line has no mapping colon).
bool split_key(const std::string &t, std::string &key, std::string &rest) {
    char q = 0;
    for (size_t i = 0; i < t.size(); ++i) {
        const char c = t[i];
        if (q) { if (c == q) q = 0; continue; }
        if (c == '"' || c == '\'') q = c;
        else if (c == '[') return false;
        else if (c == ':' && (i + 1 == t.size() || t[i + 1] == ' ' || t[i + 1] == '\t')) {
            key = trim(t.substr(0, i));
            if (key.size() >= 2 && (key.front() == '"' || key.front() == '\'')) key = key.substr(1, key.size() - 2);
            rest = t.substr(i + 1);
            return true;
        }
    }
    return false;
}

struct Parser {
    std::vector<YLine> lines;
    size_t pos = 0;
    bool ok = true;
    std::string err;

    void fail_at(const std::string &m) {
        if (ok) { ok = false; err = m + " (line " + std::to_string(pos + 1) + ")"; }
    }

    // The block starting at lines[pos] with indentation 'ind'.
    YPtr block(int ind) {
        if (pos >= lines.size() || lines[pos].indent < ind) return std::make_shared<YNode>();
        const bool seq = lines[pos].text.rfind("- ", 0) == 0 || lines[pos].text == "-";
        auto n = std::make_shared<YNode>();
        n->kind = seq ? YNode::Seq : YNode::Map;
        while (ok && pos < lines.size() && lines[pos].indent == ind) {
            const std::string t = lines[pos].text;
            if (seq) {
                if (t.rfind("-", 0) != 0) { fail_at("mapping key inside a sequence"); break; }
                std::string rest = t.size() > 1 ? t.substr(2) : std::string();
                std::string key, val;
                if (!trim(rest).empty() && split_key(rest, key, val)) {
                    // "- key: ..." : a mapping item whose keys sit in the column of 'key'
                    const int col = ind + (int)t.find_first_not_of(' ', 1);
                    lines[pos].indent = col;
                    lines[pos].text = trim(rest);
                    n->items.push_back(block(col));
                } else {
                    ++pos;
                    if (trim(rest).empty()) n->items.push_back(block_after(ind));
                    else n->items.push_back(inline_value(rest, ok));
                }
            } else {
                std::string key, val;
                if (!split_key(t, key, val)) { fail_at("expected 'key: value'"); break; }
                ++pos;
                if (trim(val).empty()) n->fields.push_back({key, block_after(ind)});
                else n->fields.push_back({key, inline_value(val, ok)});
            }
        }
        if (ok && pos < lines.size() && lines[pos].indent > ind) fail_at("unexpected indentation");
        return n;
    }

    // The nested block after a line at indentation 'ind' (null when none).
    YPtr block_after(int ind) {
        if (pos < lines.size() && lines[pos].indent > ind) return block(lines[pos].indent);
        if (pos < lines.size() && lines[pos].indent == ind && lines[pos].text.rfind("- ", 0) == 0)
            return block(ind);   // a sequence at the key's own indentation
        return std::make_shared<YNode>();
    }
};

int parse_yaml(const std::string &text, YPtr &root) {
    Parser p;
    std::stringstream ss(text);
    std::string raw;
    while (std::getline(ss, raw)) {
        for (char &c : raw) if (c == '\t') c = ' ';
        const std::string s = strip_comment(raw);
        const std::string t = trim(s);
        if (t.empty() || t == "---") continue;
        p.lines.push_back({(int)s.find_first_not_of(' '), t});
    }
    root = p.block(p.lines.empty() ? 0 : p.lines[0].indent);
    if (p.ok && p.pos < p.lines.size()) p.fail_at("text after the document");
    if (!p.ok) return fail(RPM_ERR_INVALID, "YAML: %s", p.err.c_str());
    return RPM_OK;
}

int read_file(const char *path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(RPM_ERR_INVALID, "cannot open %s", path);
    std::stringstream b;
    b << f.rdbuf();
    out = b.str();
    return RPM_OK;
}

bool as_float(const YNode *n, float &v) {
    if (!n || n->kind != YNode::Scalar) return false;
    char *end = nullptr;
    v = std::strtof(n->text.c_str(), &end);
    return end && *end == '\0' && end != n->text.c_str();
}

bool as_int(const YNode *n, int &v) {
    float f;
    if (!as_float(n, f) || f != std::floor(f)) return false;
    v = (int)f;
    return true;
}

bool as_floats(const YNode *n, float *out, int count) {
    if (!n || n->kind != YNode::Seq || (int)n->items.size() < count) return false;
    for (int k = 0; k < count; ++k)
        if (!as_float(n->items[k].get(), out[k])) return false;
    return true;
}

}  // namespace
}  // namespace impl
}  // namespace rpm

using namespace rpm::impl;

extern "C" {

int rpm_scenario_read(const char *path, rpm_scenario_info *info, float *aabb_out, float *tol_out, uint8_t *flags_out,
                      int32_t capacity) {
    if (!path || !info) return fail(RPM_ERR_INVALID, "NULL argument");
    std::string text;
    int rc = read_file(path, text);
    if (rc) return rc;
    YPtr root;
    rc = parse_yaml(text, root);
    if (rc) return rc;
    std::memset(info, 0, sizeof *info);
    const YNode *robot = root->get("robot"), *envn = root->get("environment");
    if (!robot || robot->kind != YNode::Map) return fail(RPM_ERR_INVALID, "%s: no 'robot' mapping", path);
    const YNode *type = robot->get("type");
    if (type && type->kind == YNode::Scalar) std::snprintf(info->type, sizeof info->type, "%s", type->text.c_str());
    int v = 0;
    if (as_int(robot->get("num_DOFs"), v)) info->num_dofs = v;
    // Environment.cpp:68-74: ground_included, required for the xArm6
    info->ground_included = 0;
    if (as_int(robot->get("ground_included"), v)) info->ground_included = v;
    const YNode *radii = robot->get("capsules_radius");
    if (radii && radii->kind == YNode::Seq) {
        info->num_radii = (int32_t)std::min<size_t>(radii->items.size(), RPM_MAX_DOF);
        for (int k = 0; k < info->num_radii; ++k)
            if (!as_float(radii->items[k].get(), info->capsules_radius[k]))
                return fail(RPM_ERR_INVALID, "%s: bad capsules_radius", path);
    }
    float f;
    if (as_float(robot->get("gripper_length"), f)) info->gripper_length = f;
    as_floats(robot->get("WS_center"), info->ws_center, 3);
    if (as_float(robot->get("WS_radius"), f)) info->ws_radius = f;
    if (info->num_dofs > 0 && info->num_dofs <= RPM_MAX_DOF) {
        as_floats(robot->get("q_start"), info->q_start, info->num_dofs);
        as_floats(robot->get("q_goal"), info->q_goal, info->num_dofs);
    }
    const double maxd = 1000.0;   // RealVectorSpaceConfig::MAX_DISTANCE (Box.cpp:13)
    int32_t n = 0;
    if (envn && envn->kind == YNode::Seq) {
        for (size_t i = 0; i < envn->items.size(); ++i) {
            const YNode *it = envn->items[i].get();
            const YNode *box = it ? it->get("box") : nullptr;
            if (!box) {
                if (it && it->get("sphere")) continue;   // spheres are never constructed (Environment.cpp:53-56)
                return fail(RPM_ERR_INVALID, "%s: environment item %zu is not a box", path, i);
            }
            std::string label;
            if (const YNode *l = box->get("label"); l && l->kind == YNode::Scalar) label = l->text;
            if (label == "ground" && info->ground_included == 0) continue;   // Environment.cpp:31-32
            float dim[3], posv[3], quat[4] = {0.f, 0.f, 0.f, 1.f};
            if (!as_floats(box->get("dim"), dim, 3) || !as_floats(box->get("pos"), posv, 3))
                return fail(RPM_ERR_INVALID, "%s: box %zu needs dim and pos", path, i);
            if (box->get("rot") && !as_floats(box->get("rot"), quat, 4))
                return fail(RPM_ERR_INVALID, "%s: box %zu has a bad rot", path, i);
            if (n < capacity) {
                if (aabb_out) rpm_box_aabb(dim, posv, quat, aabb_out + 6 * (size_t)n);
                float tol = (float)maxd;
                if (box->get("min_dist_tol") && !as_float(box->get("min_dist_tol"), tol))
                    return fail(RPM_ERR_INVALID, "%s: box %zu has a bad min_dist_tol", path, i);
                if (tol_out) tol_out[n] = tol;
                if (flags_out)
                    flags_out[n] = (uint8_t)((label == "ground" ? RPM_OBS_GROUND : 0u) |
                                             (label == "dynamic_obstacle" ? RPM_OBS_DYNAMIC : 0u));
            }
            ++n;
        }
    }
    info->num_obstacles = n;
    return RPM_OK;
}

int rpm_random_scenario_read(const char *path, int32_t num_obstacles, int32_t run, int32_t num_dofs, float *start,
                             float *goal, float *pos, float *vel) {
    if (!path || num_obstacles < 0 || run < 0 || num_dofs < 1 || num_dofs > RPM_MAX_DOF || !start || !goal ||
        (num_obstacles > 0 && (!pos || !vel)))
        return fail(RPM_ERR_INVALID, "bad arguments");
    std::string text;
    int rc = read_file(path, text);
    if (rc) return rc;
    YPtr root;
    rc = parse_yaml(text, root);
    if (rc) return rc;
    const YNode *sc = root->get("scenario_" + std::to_string(num_obstacles));
    const YNode *r = sc ? sc->get("run_" + std::to_string(run)) : nullptr;
    if (!r) return fail(RPM_ERR_INVALID, "%s: no scenario_%d / run_%d", path, num_obstacles, run);
    if (!as_floats(r->get("start"), start, num_dofs) || !as_floats(r->get("goal"), goal, num_dofs))
        return fail(RPM_ERR_INVALID, "%s: run %d needs start and goal of %d values", path, run, num_dofs);
    for (int j = 0; j < num_obstacles; ++j) {
        const YNode *o = r->get("object_" + std::to_string(j));
        if (!o || !as_floats(o->get("pos"), pos + 3 * j, 3) || !as_floats(o->get("vel"), vel + 3 * j, 3))
            return fail(RPM_ERR_INVALID, "%s: run %d object_%d needs pos and vel", path, run, j);
    }
    return RPM_OK;
}

// ---- the reference's robots ------------------------------------------------
// Joint tables of the URDFs under data/ as kdl_parser chains them: joint k is
// its fixed origin (xyz, rpy -> quaternion -> rotation) then a revolute joint
// about one axis of its frame; entry D is the fixed tool joint.
namespace {

// URDF rpy (fixed axes x, y, z) -> unit quaternion -> row-major rotation.
void rpy_rotation(double roll, double pitch, double yaw, double *m) {
    const double sphi = std::sin(roll / 2.0), cphi = std::cos(roll / 2.0);
    const double sthe = std::sin(pitch / 2.0), cthe = std::cos(pitch / 2.0);
    const double spsi = std::sin(yaw / 2.0), cpsi = std::cos(yaw / 2.0);
    double x = sphi * cthe * cpsi - cphi * sthe * spsi;
    double y = cphi * sthe * cpsi + sphi * cthe * spsi;
    double z = cphi * cthe * spsi - sphi * sthe * cpsi;
    double w = cphi * cthe * cpsi + sphi * sthe * spsi;
    const double n = std::sqrt(x * x + y * y + z * z + w * w);
    x /= n; y /= n; z /= n; w /= n;
    const double x2 = x * x, y2 = y * y, z2 = z * z, w2 = w * w;
    const double r[9] = {w2 + x2 - y2 - z2, 2 * x * y - 2 * w * z, 2 * x * z + 2 * w * y,
                         2 * x * y + 2 * w * z, w2 - x2 + y2 - z2, 2 * y * z - 2 * w * x,
                         2 * x * z - 2 * w * y, 2 * y * z + 2 * w * x, w2 - x2 - y2 + z2};
    std::memcpy(m, r, sizeof r);
}

void identity_rotation(double *m) {
    const double r[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::memcpy(m, r, sizeof r);
}

constexpr double kPiUrdf = 3.14159;                 // joint limits of the planar and spatial URDFs
constexpr double kPiXarm = 3.14159265359;           // joint limits of xarm6.urdf

}  // namespace

extern "C" int rpm_robot_builtin(const char *type, rpm_robot_desc *out) {
    if (!type || !out) return fail(RPM_ERR_INVALID, "NULL argument");
    rpm_robot_desc d;
    std::memset(&d, 0, sizeof d);
    const std::string t(type);
    if (t == "2dof" || t == "planar_2dof" || t == "10dof" || t == "planar_10dof") {
        // data/planar_2dof/planar_2dof.urdf, data/planar_10dof/planar_10dof.urdf: z axes, links of 1 m / 0.2 m
        const bool two = t == "2dof" || t == "planar_2dof";
        const int D = two ? 2 : 10;
        const double len = two ? 1.0 : 0.2;
        d.kind = RPM_ROBOT_CHAIN;
        d.num_dofs = D;
        for (int k = 0; k <= D; ++k) {
            d.origin_xyz[k][0] = k == 0 ? 0.0 : len;
            identity_rotation(d.origin_rot[k]);
        }
        for (int k = 0; k < D; ++k) {
            d.joint_axis[k] = 2;
            d.limits[k][0] = (float)-kPiUrdf;
            d.limits[k][1] = (float)kPiUrdf;
            d.capsule_radius[k] = 0.025f;   // URDF link box dim.y / 2 (Planar2DOF.cpp:51)
        }
    } else if (t.rfind("spatial_", 0) == 0) {
        // data/spatial_{10,14,18,22}dof/*.urdf: joint 1 about z at the base, the
        // rest about x, 0.1 m then h apart; the tool h beyond the last joint
        int D = 0;
        double h = 0;
        if (t == "spatial_10dof") { D = 10; h = 0.1; }
        else if (t == "spatial_14dof") { D = 14; h = 0.0692; }
        else if (t == "spatial_18dof") { D = 18; h = 0.05294; }
        else if (t == "spatial_22dof") { D = 22; h = 0.042857; }
        else return fail(RPM_ERR_INVALID, "unknown robot type '%s'", type);
        d.kind = RPM_ROBOT_SPATIAL;
        d.num_dofs = D;
        for (int k = 0; k <= D; ++k) {
            d.origin_xyz[k][2] = k == 0 ? 0.0 : (k == 1 ? 0.1 : h);
            identity_rotation(d.origin_rot[k]);
        }
        for (int k = 0; k < D; ++k) {
            d.joint_axis[k] = k == 0 ? 2 : 0;
            d.limits[k][0] = (float)-kPiUrdf;
            d.limits[k][1] = (float)kPiUrdf;
            d.capsule_radius[k] = 0.025f;
        }
    } else if (t == "xarm6") {
        // data/xarm6/xarm6.urdf joint1..joint6 (xyz, rpy as written, limits); the
        // capsule radii, gripper and ground rule come from the scenario
        static const double xyz[6][3] = {{0, 0, 0.267}, {0, 0, 0}, {0.0535, -0.2845, 0},
                                         {0.0775, 0.3425, 0}, {0, 0, 0}, {0.076, 0.097, 0}};
        static const double rpy[6][3] = {{0, 0, 0}, {-1.5708, 0, 0}, {0, 0, 0},
                                         {-1.5708, 0, 0}, {1.5708, 0, 0}, {-1.5708, 0, 0}};
        static const double lim[6][2] = {{-kPiXarm, kPiXarm}, {-2.059, 2.0944}, {-3.927, 0.19198},
                                         {-kPiXarm, kPiXarm}, {-1.69297, kPiXarm}, {-kPiXarm, kPiXarm}};
        d.kind = RPM_ROBOT_XARM6;
        d.num_dofs = 6;
        for (int k = 0; k < 6; ++k) {
            for (int i = 0; i < 3; ++i) d.origin_xyz[k][i] = xyz[k][i];
            rpy_rotation(rpy[k][0], rpy[k][1], rpy[k][2], d.origin_rot[k]);
            d.joint_axis[k] = 2;
            d.limits[k][0] = (float)lim[k][0];
            d.limits[k][1] = (float)lim[k][1];
        }
        identity_rotation(d.origin_rot[6]);
    } else {
        return fail(RPM_ERR_INVALID, "unknown robot type '%s'", type);
    }
    *out = d;
    return RPM_OK;
}

}  // extern "C"
