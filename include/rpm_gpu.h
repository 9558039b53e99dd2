/*
 * rpm_gpu.h -- C ABI of the GB300 collision and distance engine for
 * RPMPLv2's RealVectorSpace path.
 *
 * The engine replaces the link x obstacle loops behind
 *   base::RealVectorSpace::isValid(q)              src/state_spaces/real_vector_space/RealVectorSpace.cpp:277-309
 *   base::RealVectorSpace::isValid(q1, q2)         RealVectorSpace.cpp:261-275 (+ interpolateEdge :75-88)
 *   base::RealVectorSpace::computeDistance(q, ..)  RealVectorSpace.cpp:318-392
 * and the forward kinematics / skeleton recipes they call
 *   robots::xArm6::computeForwardKinematics/computeSkeleton    src/robots/xArm6.cpp:107-134, 209-235
 *   robots::Planar2DOF::computeForwardKinematics/computeSkeleton src/robots/Planar2DOF.cpp:82-130
 * Obstacles reach the path as fcl world AABBs (src/environments/objects/Box.cpp:3-14).
 *
 * Conventions: every entry point returns an int status (RPM_OK == 0, negative
 * on error) and never throws.  rpm_last_error_string() returns a message for
 * the last failing call on the calling thread.  Pointers named *_dev are
 * device pointers owned by the caller; pointers named *_host are ordinary or
 * pinned host pointers owned by the caller.  Robots and scenes are owned by
 * the context.  A context may be used from several host threads as long as
 * each thread passes its own stream.
 */
#ifndef RPM_GPU_H
#define RPM_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RPM_MAX_DOF 32

enum rpm_status_code {
    RPM_OK = 0,
    RPM_ERR_INVALID = -1,     /* bad argument, unknown handle, unsupported robot */
    RPM_ERR_CUDA = -2,        /* a CUDA runtime call failed */
    RPM_ERR_NOMEM = -3,       /* device or pinned allocation failed */
    RPM_ERR_TIMEOUT = -4,     /* a bounded device-side wait gave up */
    RPM_ERR_ADMISSION = -5,   /* request rejected by the memory budget */
    RPM_ERR_RANGE = -6        /* size beyond a stated maximum */
};

/* Robot families of the reference.  CHAIN is robots::Planar2DOF and
 * Planar10DOF, SPATIAL is robots::Spatial10DOF and the Spatial14/18/22DOF
 * classes derived from it: for both, skeleton point k is the origin of chain
 * segment k, k = 0..D (Planar2DOF.cpp:125-126); they differ only in
 * computeEnclosingRadii (Spatial10DOF.cpp:11-30 projects row 0 on {x, y}).
 * XARM6 is robots::xArm6 with its 7-point skeleton recipe and gripper offset
 * (xArm6.cpp:130, 215-231). */
enum rpm_robot_kind { RPM_ROBOT_CHAIN = 0, RPM_ROBOT_XARM6 = 1, RPM_ROBOT_SPATIAL = 2 };

/* Kinematic description of a serial chain as kdl_parser builds it from the
 * URDF: joint k (0-based) has a fixed origin (origin_xyz[k], origin_rot[k])
 * in its parent frame followed by a revolute rotation q_k about the unit axis
 * joint_axis[k] (0 = x, 1 = y, 2 = z) of the joint frame.  Entry D of the
 * origin arrays is the fixed tool joint ("ee" / "joint_eef").  origin_rot is
 * row-major and is used as given, so the URDF rpy values (e.g. -1.5708, not
 * -pi/2) are preserved. */
typedef struct rpm_robot_desc {
    int32_t kind;                          /* enum rpm_robot_kind */
    int32_t num_dofs;                      /* D; also the number of capsule links */
    int32_t ground_included;               /* links i < ground_included ignore "ground" obstacles */
    float   gripper_length;                /* XARM6 only (xArm6.cpp:130, 231) */
    int32_t joint_axis[RPM_MAX_DOF];
    double  origin_xyz[RPM_MAX_DOF + 1][3];
    double  origin_rot[RPM_MAX_DOF + 1][9];
    float   capsule_radius[RPM_MAX_DOF];   /* AbstractRobot::getCapsuleRadius(i) */
    float   limits[RPM_MAX_DOF][2];        /* joint limits (lower, upper); informational */
} rpm_robot_desc;

/* Obstacle flags (per obstacle). */
#define RPM_OBS_GROUND  0x1u   /* label == "ground": skipped for links i < ground_included (RealVectorSpace.cpp:285, 336) */
#define RPM_OBS_DYNAMIC 0x2u   /* label == "dynamic_obstacle" (moved by incremental updates) */

/* RealVectorSpaceConfig constants as the YAML sets them
 * (data/configurations/configuration_realvectorspace.yaml:1-3). */
typedef struct rpm_params {
    double equality_threshold;   /* EQUALITY_THRESHOLD, 1e-4 */
    double max_distance;         /* MAX_DISTANCE, 1000 */
} rpm_params;

/* Arithmetic forms of the check. */
enum rpm_precision {
    RPM_PREC_FP64 = 0,          /* FP64 FK and narrow phase ("plain form") */
    RPM_PREC_FP32_RECHECK = 1,  /* FP32 bulk pass; configs near any decision boundary are recomputed in FP64 */
    RPM_PREC_FP32_REF = 2       /* the reference's own numerics: FP64 FK rounded to FP32, FP32 narrow phase */
};

/* How configuration checks are spread over the GPU.  Results are identical. */
enum rpm_layout {
    RPM_LAYOUT_AUTO = 0,        /* chosen per segment from the scene size, link count and batch size */
    RPM_LAYOUT_LANE = 1,        /* one lane per configuration, obstacles walked in order */
    RPM_LAYOUT_WARP = 2         /* one warp per configuration over the spatially sorted obstacles */
};

typedef struct rpm_ctx rpm_ctx;

/* Statistics of the last check issued on a context (read after a sync). */
typedef struct rpm_check_stats {
    int64_t configs;           /* configurations (or edge checks) in the call */
    int64_t rechecked;         /* FP64 rechecks of the call: configurations recomputed whole or through their
                                  listed pairs, once per output pass (isValid, distance) that needed one */
    int64_t overflow;          /* recheck entries that did not fit the recheck list (must be 0) */
    int32_t device_status;     /* 0, or an RPM_ERR_* recorded by a kernel */
    int32_t pad;
} rpm_check_stats;

/* ---- errors ---------------------------------------------------------------- */
const char *rpm_last_error_string(void);
int rpm_version(void);

/* ---- context ----------------------------------------------------------------
 * Replaces nothing in the reference (it has no device); holds the device
 * robots, scenes and reusable scratch. */
int rpm_ctx_create(int device, rpm_ctx **out);
int rpm_ctx_destroy(rpm_ctx *ctx);
int rpm_ctx_set_params(rpm_ctx *ctx, const rpm_params *params);

/* ---- robots -----------------------------------------------------------------
 * Replaces the robot construction from URDF (xArm6.cpp:7-76, Planar2DOF.cpp:7-64,
 * Spatial10DOF.cpp:5-9) plus AbstractRobot::setCapsulesRadius / setGroundIncluded. */
int rpm_robot_upload(rpm_ctx *ctx, const rpm_robot_desc *desc, int32_t *robot_id);
/* The kinematic table of one of the reference's robots by its type name, as
 * robots::AbstractRobot::getType() returns it (the URDF robot name): "2dof",
 * "10dof" (also "planar_2dof", "planar_10dof"), "spatial_10dof",
 * "spatial_14dof", "spatial_18dof", "spatial_22dof", "xarm6" -- the joint
 * origins, axes and limits of data/<robot>/<robot>.urdf as kdl_parser chains
 * them (Planar2DOF.cpp:7-64, Spatial10DOF.cpp:5-9, xArm6.cpp:7-76).  Capsule
 * radii default to the URDF link boxes' dim.y / 2 (0.025; 0 for xarm6, whose
 * radii come from the scenario), ground_included and gripper_length to 0: a
 * caller overrides them from its robot (setCapsulesRadius, setGroundIncluded,
 * setGripperLength).  Host only. */
int rpm_robot_builtin(const char *type, rpm_robot_desc *out);

/* ---- scenes (device-resident obstacle sets) ----------------------------------
 * Replaces env::Environment's object list as the hot path sees it
 * (Environment.cpp:13-56; fcl AABB per Box.cpp:6-7).  aabb_host is n x 6
 * floats (xmin, ymin, zmin, xmax, ymax, zmax) per obstacle, exactly the
 * 'obs' vector of RealVectorSpace.cpp:293-295; min_dist_tol_host is
 * Object::getMinDistTol (Box.cpp:13, YAML min_dist_tol); flags_host holds
 * RPM_OBS_* bits.  min_dist_tol_host and flags_host may be NULL (MAX_DISTANCE, 0).
 * A scene holds at most RPM_MAX_OBSTACLES obstacles (RPM_ERR_RANGE beyond). */
#define RPM_MAX_OBSTACLES 2048
int rpm_scene_create(rpm_ctx *ctx, int32_t robot_id, const float *aabb_host, const float *min_dist_tol_host,
                     const uint8_t *flags_host, int32_t n, int32_t *scene_id);
/* Replace the AABBs of obstacles idx[0..m) (Object::setPosition, Object.cpp:21-26;
 * Environment::updateEnvironment moves).  Incremental and asynchronous: the
 * next version is the current one copied on the device with the m rows
 * scattered in.  It is visible to every check issued on any stream after this
 * call returns; checks already issued keep the version they started with. */
int rpm_scene_update(rpm_ctx *ctx, int32_t scene_id, const int32_t *idx_host, const float *aabb_host, int32_t m,
                     uint64_t *version_out);
/* rpm_scene_update for several scenes at once (each at most once): scene k
 * takes counts[k] rows, consecutive in idx_host (indices) and aabb_host (six
 * floats each).  All the new versions are written by one launch, so moving the
 * dynamic obstacles of many scenes every few milliseconds (the reference's
 * Environment::updateEnvironment per environment) costs one update.
 * versions_out[k] (nullable) receives scene k's new version. */
int rpm_scene_update_many(rpm_ctx *ctx, int32_t n_scenes, const int32_t *scene_ids, const int32_t *counts,
                          const int32_t *idx_host, const float *aabb_host, uint64_t *versions_out);
int rpm_scene_destroy(rpm_ctx *ctx, int32_t scene_id);
int rpm_scene_info(rpm_ctx *ctx, int32_t scene_id, int32_t *robot_id, int32_t *num_obstacles, uint64_t *version);

/* fcl 0.7 world AABB of a box (Box.cpp:6-7): identity rotation gives
 * pos +- dim/2; any other rotation gives the cube pos +- |dim/2|. */
int rpm_box_aabb(const float dim[3], const float pos[3], const float quat_xyzw[4], float aabb_out[6]);

/* ---- batched checks ------------------------------------------------------------
 * For configurations q_dev (C x D floats, row-major, one RealVectorSpaceState
 * coordinate vector per row) compute
 *   valid_dev[c]   = isValid(q_c)                     (1 valid, 0 in collision)  nullable
 *   dist_dev[c]    = computeDistance(q_c, true)        (0 on collision)          nullable
 *   profile_dev[c*L+i] = d_c_profile[i] after computeDistance, including its
 *                    early-exit shape (RealVectorSpace.cpp:370-378)            nullable
 * All work is queued on 'stream' (a cudaStream_t, NULL = legacy default). */
int rpm_check_configs(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev, int64_t num_configs,
                      uint8_t *valid_dev, double *dist_dev, float *profile_dev, void *stream);

/* Several scenes (and robots of different DOF) in one launch: item k checks
 * num_configs configurations of its own scene (mixed-DOF batches of
 * spatial 14/18/22-DOF robots, serving batches).  Same outputs as
 * rpm_check_configs per item. */
typedef struct rpm_batch_item {
    int32_t scene_id;
    int32_t reserved;
    const float *q_dev;       /* num_configs x D of the scene's robot */
    int64_t num_configs;
    uint8_t *valid_dev;       /* nullable */
    double *dist_dev;         /* nullable */
    float *profile_dev;       /* nullable, num_configs x L */
} rpm_batch_item;
int rpm_check_batch(rpm_ctx *ctx, int32_t precision, const rpm_batch_item *items, int32_t n_items, void *stream);

/* Same as rpm_check_configs with host buffers; returns after the results are
 * in the host buffers.  When every buffer is page-locked host memory
 * (cudaHostAlloc / cudaHostRegister), the kernels read the configurations and
 * write the outputs there directly (over NVLink-C2C on GB300) in one launch,
 * unless the batch is one the FP32 + recheck lane kernel checks in binned
 * order (at least 2,048 configurations); that batch, and any batch in other
 * buffers, is staged in chunks through context-owned device memory, with the
 * copies overlapping the checks. */
int rpm_check_configs_host(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_host, int64_t num_configs,
                           uint8_t *valid_host, double *dist_host, float *profile_host);

/* RealVectorSpace::isValid(q1, q2) (RealVectorSpace.cpp:261-275) for a batch
 * of edges (q1_dev, q2_dev: E x D).  With step > 0 edge e is checked at
 * n_e = max(1, ceil(|q1 - q2| / step)) points, otherwise at num_checks points
 * (NUM_INTERPOLATION_VALIDITY_CHECKS); points run from q2 towards q1 as in the
 * reference and q1 itself is not checked.  valid_dev[e] = isValid(q1, q2);
 * checks_dev[e] (nullable) = the number of checks the reference evaluates
 * before its early exit.  Runs as a persistent work-queue kernel; with
 * rpm_ctx_set_graphs enabled, repeated calls with the same arguments replay
 * a captured CUDA graph of the whole pipeline. */
int rpm_check_edges(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q1_dev, const float *q2_dev,
                    int64_t num_edges, float step, int32_t num_checks, uint8_t *valid_dev, int32_t *checks_dev,
                    void *stream);
int rpm_ctx_set_graphs(rpm_ctx *ctx, int enable);
/* rpm_check_edges for several edge sets in one pipeline: each item has its
 * own scene (and so robot, DOF count and obstacles), edges, discretisation
 * and outputs, as rpm_check_edges.  Items are checked together (the
 * batching form for uneven discretisations and mixed-DOF robots); each
 * item's outputs equal what rpm_check_edges gives for it alone. */
typedef struct rpm_edge_batch_item {
    int32_t scene_id;
    int32_t num_checks;
    int64_t num_edges;
    const float *q1_dev;      /* num_edges x D of the scene's robot */
    const float *q2_dev;
    float step;
    uint8_t *valid_dev;
    int32_t *checks_dev;      /* nullable */
} rpm_edge_batch_item;
int rpm_check_edges_batch(rpm_ctx *ctx, int32_t precision, const rpm_edge_batch_item *items, int32_t n_items,
                          void *stream);
/* ---- tile shapes and the autotuner -------------------------------------------
 * A GB300 addition with no reference counterpart; results never depend on
 * the shape, only the time does.  A tile shape is how a batch is spread over
 * the GPU: the layout (one lane per configuration or edge check, or one warp
 * per configuration over the scene sorted into leaves), the configurations
 * (or edge streams) each warp of the warp layout takes, and the persistent
 * CTAs per SM of the lane-layout edge pass.  The context keeps a table of
 * shapes per bucket (robot kind and DOF, obstacles and batch size as
 * ceil(log2), precision, outputs, configurations or edges); a bucket without
 * an entry takes the built-in rule (RPM_LAYOUT_AUTO).  The table is used only
 * in RPM_LAYOUT_AUTO. */
typedef struct rpm_tile_shape {
    int32_t layout;             /* RPM_LAYOUT_LANE or RPM_LAYOUT_WARP (0: the built-in rule) */
    int32_t configs_per_warp;   /* warp layout: configurations or edge streams per warp; 0: chosen by size */
    int32_t ctas_per_sm;        /* lane-layout edge pass: persistent CTAs per SM; 0: 4 */
    float ms;                   /* the time the autotuner measured for the bucket's call (0 if set by hand) */
} rpm_tile_shape;
/* Outputs of a bucket: bit 0 isValid, bit 1 distance, bit 2 profile (edges: 1). */
#define RPM_OUT_VALID   0x1
#define RPM_OUT_DIST    0x2
#define RPM_OUT_PROFILE 0x4
/* Time rpm_check_configs on the given batch (outputs as given: nullable) in
 * every candidate shape -- the lane layout, and the warp layout with 1, 2, 4,
 * 8, 16 or 32 configurations per warp (up to what the warp's skeleton buffer
 * holds for the robot, and that bound itself) and the size rule -- each 'reps' times
 * after a warm-up (median), and keep the fastest for the batch's bucket;
 * *best receives it. */
int rpm_autotune_configs(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev, int64_t num_configs,
                         uint8_t *valid_dev, double *dist_dev, float *profile_dev, int32_t reps, rpm_tile_shape *best);
/* The same for rpm_check_edges: the lane layout with 1, 2, 3, 4, 6 or 8
 * persistent CTAs per SM, and the warp layout with the size rule or 1, 2, 4,
 * 8 edge streams per warp. */
int rpm_autotune_edges(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q1_dev, const float *q2_dev,
                       int64_t num_edges, float step, int32_t num_checks, uint8_t *valid_dev, int32_t reps,
                       rpm_tile_shape *best);
/* Set (shape non-NULL) or remove (NULL) the entry of the bucket of this
 * scene, precision, kind (edges 0/1), batch size and outputs. */
int rpm_set_tile_shape(rpm_ctx *ctx, int32_t scene_id, int32_t precision, int32_t edges, int64_t count,
                       int32_t outputs, const rpm_tile_shape *shape);
/* The table as a JSON file (one entry per line), and back: loading adds or
 * replaces entries.  A context created while RPM_TUNING_FILE names a file
 * loads it. */
int rpm_tuning_save(rpm_ctx *ctx, const char *path);
int rpm_tuning_load(rpm_ctx *ctx, const char *path);
/* The shape of the last configuration or edge launch issued on 'stream'. */
int rpm_last_shape(rpm_ctx *ctx, void *stream, rpm_tile_shape *out);
/* Layout of the configuration checks (rpm_check_configs, rpm_check_batch,
 * rpm_check_configs_host and the server): one of enum rpm_layout.  A GB300
 * addition with no reference counterpart; outputs do not depend on it. */
int rpm_ctx_set_layout(rpm_ctx *ctx, int32_t layout);

/* computeDistance(q, true) with the nearest points (RealVectorSpace.cpp:318-392)
 * for the single-state adapter path: every (link, obstacle) pair is evaluated.
 * dist_dev[c] (double); profile_dev[c][L] (float, the early-exit profile);
 * nearest_dev[c][n][6][L] (float; rows 0-2 the robot point, rows 3-5 the
 * obstacle point, one column per link: the reference's vector<MatrixXf(6, L)>);
 * nearest_valid_dev[c] = 0 where the reference sets the nearest points to
 * nullptr (some link at distance <= 0).  precision RPM_PREC_FP64 or
 * RPM_PREC_FP32_REF (bit-equal to the reference's numerics);
 * RPM_PREC_FP32_RECHECK is served by the FP64 form. */
int rpm_distance_nearest(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev, int64_t num_configs,
                         double *dist_dev, float *profile_dev, float *nearest_dev, uint8_t *nearest_valid_dev,
                         void *stream);
/* computeDistanceUnderestimation (RealVectorSpace.cpp:402-446): per link, the
 * smallest distance of its skeleton points to the planes through the obstacle
 * points O of nearest_dev (layout as above) with normals (R - O)/|R - O|,
 * minus the radius.  complete_dev[c] = 0 where the reference returns 0 at the
 * first negative value without updating the state (dist 0, profile not
 * written); otherwise dist_dev[c] and profile_dev[c][L] are the reference's
 * d_c and profile.  Same precisions as rpm_distance_nearest. */
int rpm_distance_underestimation(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev,
                                 int64_t num_configs, const float *nearest_dev, double *dist_dev, float *profile_dev,
                                 uint8_t *complete_dev, void *stream);

/* How close each configuration's answers lie to a decision boundary of the
 * reference's trees (RealVectorSpace.cpp:277-309, 318-392 with
 * CollisionAndDistance.cpp:4-755), in metres over the error amplification of
 * the compared quantities, evaluated in FP64 on the FP64 skeleton.  The
 * isValid margin is that of the OR over the pairs (a collision as robust as
 * its most robust colliding pair, a free configuration as its least robust
 * pair); the distance margin is the smallest among the pairs that can set d_c
 * (within 1e-3 m of it), including the contact band and min_dist_tol rules,
 * or for a collision the largest among the pairs at distance 0.  Where the
 * reference's FP32 numerics and FP64 disagree on a configuration, its margin
 * lies inside the FP32 rounding band (about 1e-5 m): the diagnostic that
 * explains such flips. */
int rpm_decision_margins(rpm_ctx *ctx, int32_t scene_id, const float *q_dev, int64_t num_configs,
                         double *margin_valid_dev, double *margin_dist_dev, void *stream);

/* Skeleton points (L+1 points x 3) per configuration, widened to double
 * (computeSkeleton; xArm6.cpp:209-235, Planar2DOF.cpp:117-130): RPM_PREC_FP64
 * gives the FP64 points, RPM_PREC_FP32_REF the reference's float skeleton,
 * RPM_PREC_FP32_RECHECK the FP32 FK of the bulk pass. */
int rpm_skeleton(rpm_ctx *ctx, int32_t robot_id, int32_t precision, const float *q_dev, int64_t num_configs,
                 double *points_dev, void *stream);

/* ---- bubbles and spines (the RBT planners' step after the distance profile)
 * All in the reference's float numerics (its float skeleton, IEEE float
 * operations); xArm6 self-collision checking is off.  Status values are
 * base::State::Status (State.h:22). */
enum rpm_state_status { RPM_STATE_NONE = 0, RPM_STATE_ADVANCED = 1, RPM_STATE_TRAPPED = 2, RPM_STATE_REACHED = 3 };

/* AbstractRobot::computeEnclosingRadii (xArm6.cpp:237-275, Spatial10DOF.cpp:11-30,
 * Planar2DOF.cpp:132-148) for a batch: radii_dev[c] is the D x (D + 1)
 * matrix R, row-major (R[i][j]: the radius about joint i enclosing skeleton
 * points i+1..j and their capsules). */
int rpm_enclosing_radii(rpm_ctx *ctx, int32_t robot_id, const float *q_dev, int64_t num_configs, float *radii_dev,
                        void *stream);

/* RBTConnect::extendSpine (RBTConnect.cpp:85-150) for a batch of spines:
 * spine c runs from q_dev[c] towards q_e_dev[c] (num_spines x D), given the
 * start's d_c (dist_dev, float, as computeDistance returns it) and its
 * profile (profile_dev, num_spines x L).  num_iter = NUM_ITER_SPINE,
 * expanded = USE_EXPANDED_BUBBLE.  q_new_dev gets each spine's end and
 * status_dev its rpm_state_status. */
int rpm_extend_spines(rpm_ctx *ctx, int32_t robot_id, const float *q_dev, const float *q_e_dev, const float *dist_dev,
                      const float *profile_dev, int64_t num_spines, int32_t num_iter, int32_t expanded, float *q_new_dev,
                      int32_t *status_dev, void *stream);

/* DRGBT::computeReachedState (DRGBT.cpp:475-495) for a whole horizon in one
 * launch (the DRGBT generalized bur, DRGBT.cpp:272-320): for every horizon
 * state h, extendGenSpine (RGBTConnect.cpp:73-93) from q_current towards
 * horizon_dev[h] -- computeDistance of q_current with nearest points, then
 * up to num_layers spines, each followed by computeDistanceUnderestimation
 * from q_current's nearest points and stopped below d_crit -- then
 * computeDistance(q_reached, true) in 'precision' (dist_dev, nullable).
 * q_reached_dev is horizon_size x D; status_dev per rpm_state_status
 * (RPM_STATE_REACHED = isReached).  Working memory is a per-stream block
 * reused in stream order; the first call on a stream, or one that needs
 * more, grows it in stream order (cudaMallocAsync), without synchronising. */
typedef struct rpm_spine_params {
    int32_t num_layers;   /* RGBTConnectConfig::NUM_LAYERS */
    int32_t num_iter;     /* RBTConnectConfig::NUM_ITER_SPINE */
    int32_t expanded;     /* RBTConnectConfig::USE_EXPANDED_BUBBLE */
    float d_crit;         /* RBTConnectConfig::D_CRIT */
} rpm_spine_params;
int rpm_reached_states(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_current_dev,
                       const float *horizon_dev, int64_t horizon_size, const rpm_spine_params *params,
                       float *q_reached_dev, int32_t *status_dev, double *dist_dev, void *stream);

/* ---- motion validity with moving obstacles (DRGBT replanning) -------------
 * A box of the scene that moves during a motion, by
 * Environment::moveStraight (Environment.cpp:220-233): before each check its
 * position x decreases by delta_time * max_vel, and its AABB is recomputed as
 * fcl does for a box (rpm_box_aabb). */
typedef struct rpm_moving_box {
    int32_t index;          /* obstacle of the scene (label "dynamic_obstacle") */
    float max_vel;          /* Object::getMaxVel, m/s */
    float dim[3];
    float pos[3];           /* position when the motion starts */
    float quat_xyzw[4];
} rpm_moving_box;

/* MotionValidity::check (MotionValidity.cpp:30-53) for a batch of motions
 * q_prev_dev[m] -> q_cur_dev[m] (num_motions x D), each checked from the
 * scene's current obstacle state while the given boxes move:
 * delta_time = max_iter_time / num_points (num_points =
 * NUM_VALIDITY_POINTS_CHECK, MotionValidity.cpp:20-22); check k = 1..num_points
 * moves the boxes k steps and tests interpolateEdge(q_prev, q_cur,
 * dist * k / num_points, dist).  valid_dev[m] is the reference's result and
 * checks_dev[m] (nullable) the checks it makes (the first invalid k, or
 * num_points).  The scene itself is not changed: a caller that follows the
 * reference moves its boxes with rpm_scene_update.  precision RPM_PREC_FP64
 * or RPM_PREC_FP32_REF (the reference's numerics). */
int rpm_motion_validity(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_prev_dev,
                        const float *q_cur_dev, int64_t num_motions, const rpm_moving_box *boxes, int32_t num_boxes,
                        float max_iter_time, int32_t num_points, uint8_t *valid_dev, int32_t *checks_dev, void *stream);
/* The environment side of MotionValidity::check: 'steps' calls of
 * Environment::moveStraight(delta_time) (Environment.cpp:220-233) on the
 * given boxes -- boxes[b].pos is advanced in place, in float as the
 * reference does -- and their new AABBs written to the device scene as one
 * incremental update (rpm_scene_update; version in *version_out, nullable). */
int rpm_scene_move_straight(rpm_ctx *ctx, int32_t scene_id, rpm_moving_box *boxes, int32_t num_boxes, float delta_time,
                            int32_t steps, uint64_t *version_out);

/* ---- scene I/O (host only) -------------------------------------------------
 * The reference's scenario files.  rpm_scenario_read reads a scenario YAML
 * (data/<robot>/<scenario>/*.yaml) as Environment::Environment
 * (Environment.cpp:13-109) does: box obstacles as fcl world AABBs
 * (rpm_box_aabb of dim, pos and rot [x, y, z, w]), their min_dist_tol
 * (MAX_DISTANCE when absent) and flags (label "ground" -> RPM_OBS_GROUND,
 * "dynamic_obstacle" -> RPM_OBS_DYNAMIC; the ground is left out when
 * robot.ground_included is 0), plus the robot fields below.  Up to
 * 'capacity' obstacles are written (outputs nullable); info->num_obstacles is
 * the total, so a first call with capacity 0 sizes the arrays.  Spheres are
 * skipped (the reference never constructs them); any other object type is an
 * error. */
typedef struct rpm_scenario_info {
    char type[32];                       /* robot.type, e.g. "xarm6", "spatial_10dof" */
    int32_t num_dofs;                    /* robot.num_DOFs */
    int32_t ground_included;             /* robot.ground_included (0 when absent) */
    int32_t num_radii;                   /* entries of robot.capsules_radius (1 = broadcast) */
    int32_t num_obstacles;
    float capsules_radius[RPM_MAX_DOF];
    float gripper_length;
    float ws_center[3];
    float ws_radius;
    float q_start[RPM_MAX_DOF];
    float q_goal[RPM_MAX_DOF];
} rpm_scenario_info;
int rpm_scenario_read(const char *path, rpm_scenario_info *info, float *aabb_out, float *tol_out, uint8_t *flags_out,
                      int32_t capacity);
/* One run of a random_scenarios.yaml (apps/test_drgbt_random_obstacles.cpp:125-151):
 * scenario_<num_obstacles>/run_<run>: start and goal (num_dofs each) and, per
 * object_j, pos and vel (num_obstacles x 3 each).  The objects are boxes of
 * the scenario's random_obstacles.dim with label "dynamic_obstacle". */
int rpm_random_scenario_read(const char *path, int32_t num_obstacles, int32_t run, int32_t num_dofs, float *start,
                             float *goal, float *pos, float *vel);

/* ---- serving loop (continuous batching) -----------------------------------
 * Planners submit isValid / distance batches and edge batches of any size
 * against resident scenes while obstacles move (the DRGBT replanning shape,
 * DRGBT.cpp:79-176 with MotionValidity.cpp:30-53).  A worker thread admits
 * requests as device memory of the budget frees up and serves them in two
 * classes, each in arrival order:
 *   express  requests of at most express_work units (a configuration counts
 *            1, an edge 8) on high-priority streams; a request of 1,024 units
 *            or more runs as a batch of its own, smaller ones share batches of
 *            up to 1,024 units, so a replanning query never waits behind bulk
 *            work or behind another query;
 *   bulk     larger requests on low-priority streams, packed up to
 *            max_batch_configs units per batch and run as chains of launches
 *            of at most chunk_work units, so every bulk CTA is short and the
 *            block scheduler gives SMs to express kernels quickly.
 * A batch packs configuration and edge requests from any scenes and robots
 * into multi-segment launches; batches overlap on the device; every request
 * is time-stamped.  Host buffers should be pinned for copies to overlap.
 * Processes that set CUDA_DEVICE_MAX_CONNECTIONS to 32 before creating their
 * CUDA context (the Python package does) keep the streams on separate
 * hardware queues. */
typedef struct rpm_server rpm_server;
typedef struct rpm_server_config {
    int32_t num_slots;           /* bulk streams (concurrent bulk batches); 0: 4 */
    int32_t precision;           /* RPM_PREC_* of every request */
    int64_t memory_budget;       /* device bytes for request buffers (admission), default 8 GiB */
    int32_t max_batch_segments;  /* configuration requests and edge requests per batch, each <= 32 */
    int32_t max_batch_configs;   /* work per bulk batch; 0: 65,536 (a larger request runs as a batch of its own) */
    int32_t express_slots;       /* high-priority streams for express requests; 0: 24 */
    int32_t express_work;        /* largest express request; 0: 8,192 */
    int32_t chunk_work;          /* work per bulk launch; 0: 65,536 */
    int32_t bulk_sms;            /* > 0: the bulk streams run in an SM partition (a green context) of this
                                    many SMs (rounded up to the driver's granularity, 8 on GB300), so the
                                    other SMs only run express work; 0: all SMs but 48 where the driver
                                    offers green contexts, else every SM; -1: bulk uses every SM */
    int32_t reserved;
} rpm_server_config;

/* Request kinds: configuration checks, edge checks, and the two DRGBT
 * replanning steps (DRGBT.cpp:272-320, 475-495; MotionValidity.cpp:30-53),
 * which go through the same admission, classes and streams. */
enum rpm_request_kind { RPM_REQ_CONFIGS = 0, RPM_REQ_EDGES = 1, RPM_REQ_REACHED = 2, RPM_REQ_MOTION = 3 };

typedef struct rpm_request {
    int32_t kind;                /* enum rpm_request_kind */
    int32_t scene_id;
    int64_t count;               /* configurations or edges */
    const float *q_host;         /* CONFIGS: count x D */
    const float *q1_host;        /* EDGES: count x D each */
    const float *q2_host;
    float step;                  /* EDGES: as rpm_check_edges */
    int32_t num_checks;
    uint8_t *valid_host;         /* isValid (required for EDGES) */
    double *dist_host;           /* CONFIGS, nullable */
    float *profile_host;         /* CONFIGS, nullable */
    int32_t *checks_host;        /* EDGES, MOTION: nullable */
    /* REACHED (rpm_reached_states over a horizon of count states): q_host is
     * q_current (1 x D), q1_host the horizon (count x D); outputs q_out_host
     * (count x D), status_host (count) and dist_host (nullable; in the
     * server's precision) */
    const rpm_spine_params *spine;
    float *q_out_host;
    int32_t *status_host;
    /* MOTION (rpm_motion_validity of count motions q1_host -> q2_host while
     * the boxes move; in the reference's own numerics, or FP64 when the
     * server runs RPM_PREC_FP64): outputs valid_host, checks_host */
    const rpm_moving_box *boxes;
    int32_t num_boxes;
    int32_t num_points;
    float max_iter_time;
    int32_t reserved;
} rpm_request;

typedef struct rpm_request_timing {
    int32_t status;              /* 0 done, 1 pending, < 0 error (RPM_ERR_ADMISSION: larger than the budget) */
    int32_t batch_size;          /* requests in the launch it ran in */
    double t_submit, t_admit, t_launch, t_done;   /* seconds (monotonic; relative to the start in a replay) */
    uint64_t scene_version;      /* the version of the request's scene its checks read (rpm_scene_update) */
    /* device-side trace of the request's batch (CUDA events on its stream):
     * copies in, checks and copies out, each from the end of the previous
     * step (so a step's time includes waiting for copy engines or SMs) */
    float h2d_ms, kernel_ms, d2h_ms;
    float enqueue_ms;            /* host time the worker spent enqueueing the batch */
} rpm_request_timing;

/* A moving obstacle of a replay: AABB(t) = AABB(0) + velocity * t. */
typedef struct rpm_motion {
    int32_t scene_id;
    int32_t index;
    float velocity[3];
} rpm_motion;

int rpm_server_create(rpm_ctx *ctx, const rpm_server_config *cfg, rpm_server **out);
int rpm_server_submit(rpm_server *srv, const rpm_request *req, uint64_t *ticket);
int rpm_server_poll(rpm_server *srv, uint64_t ticket, rpm_request_timing *out);
int rpm_server_wait(rpm_server *srv, uint64_t ticket, double timeout_s, rpm_request_timing *out);
int rpm_server_release(rpm_server *srv, uint64_t ticket);
/* Submits reqs[i] at arrival_s[i] seconds after the start from a native
 * thread while a second thread moves the given obstacles every period_s
 * (incremental scene updates), waits for every request and returns their
 * timings relative to the start. */
int rpm_server_replay(rpm_server *srv, const rpm_request *reqs, const double *arrival_s, int64_t n,
                      const rpm_motion *motions, int32_t n_motions, double period_s, rpm_request_timing *out);
int rpm_server_stats(rpm_server *srv, int64_t *batches, int64_t *pending);
int rpm_server_destroy(rpm_server *srv);

/* Statistics of the last check on this context; synchronises 'stream'. */
int rpm_last_stats(rpm_ctx *ctx, void *stream, rpm_check_stats *out);

/* Per-kernel timing of later checks (CUDA events on the caller's stream).
 * rpm_last_timing returns the bulk kernel's and the recheck kernel's duration
 * of the last check on 'stream' (synchronises it). */
int rpm_ctx_set_timing(rpm_ctx *ctx, int enable);
int rpm_last_timing(rpm_ctx *ctx, void *stream, float *bulk_ms, float *recheck_ms);

/* Failure detection without a fault: launches one CTA whose shared-memory
 * staging wait can never complete (no copy is issued), bounded at 'polls'
 * polls (1 .. 2^22).  The kernel records the timeout in a status word and
 * returns, as every staging wait of the library does; the call then returns
 * RPM_ERR_TIMEOUT, and the context stays usable. */
int rpm_probe_bounded_wait(rpm_ctx *ctx, uint32_t polls);

/* The decision trees on single primitives, for parity tests against the
 * reference's own CollisionAndDistance.cpp on directed edge cases.  Case i
 * evaluates, by kind_dev[i]:
 *   0  collisionCapsuleToBox(a, b, r, aabb)    CollisionAndDistance.cpp:4-42   (value 1 = collision)
 *   1  distanceCapsuleToBox(a, b, r, aabb)     :208-214, 409-755 (d_c, radius subtracted)
 *   2  distanceLineSegToLineSeg(a, b, c, d)    :217-320
 * a_dev, b_dev: n x 3; x_dev: n x 6 (the AABB, or c then d); r_dev: n.
 * RPM_PREC_FP64 and RPM_PREC_FP32_REF evaluate the FP64 and the reference's
 * FP32 trees.  RPM_PREC_FP32_RECHECK evaluates the FP32 pass's trees with
 * their margins: settled_dev[i] = 1 where the pass settles the case, 0 where
 * it leaves it to the FP64 recheck (value_dev then holds the FP64 value, as
 * the form's outputs do), 2 if the pass's two compilations of the collision
 * tree disagree (never expected). */
int rpm_probe_primitives(rpm_ctx *ctx, int32_t precision, const int32_t *kind_dev, const float *a_dev,
                         const float *b_dev, const float *x_dev, const float *r_dev, int64_t n, double *value_dev,
                         uint8_t *settled_dev, void *stream);

/* FP32 FMA throughput of the device (TFLOP/s), measured with independent FMA
 * chains: the denominator of the FP32 roofline. */
int rpm_probe_fp32_peak(rpm_ctx *ctx, double *tflops);

/* The FP32 + FP64-recheck check of rpm_check_configs for callers that cannot
 * allocate device memory (a real-time loop that forbids allocator calls after
 * start-up, a framework that owns all device memory and hands out only its
 * own buffers).  No counterpart in the reference: it adds a calling
 * convention, not a reference operation.  Everything is passed in: the robot
 * as a host descriptor, obstacles as the caller's device arrays (aabb_dev n x 6
 * floats as in rpm_scene_create, min_dist_tol_dev and flags_dev nullable),
 * configurations and outputs as device pointers.  It calls no cudaMalloc,
 * cudaFree or allocating library routine; its scratch (the recheck list) is a
 * static device array of 65,536 entries (~512 KB held on every GPU that loads
 * the library), so num_configs above 65,536 returns RPM_ERR_RANGE.  The first
 * call on each device looks up the array's address and should come before any
 * stream capture; a call that finds another context current on the device
 * (after cudaDeviceReset) looks it up again.  All calls share the array and
 * keep the last call's contents: calls that overlap on the GPU race and must
 * be serialised by the caller. */
int rpm_check_configs_noalloc(const rpm_robot_desc *robot, const float *aabb_dev, const float *min_dist_tol_dev,
                              const uint8_t *flags_dev, int32_t n, const rpm_params *params, const float *q_dev,
                              int64_t num_configs, uint8_t *valid_dev, double *dist_dev, float *profile_dev,
                              void *stream);

/* Synchronise a stream and report any device-side error status. */
int rpm_sync(rpm_ctx *ctx, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RPM_GPU_H */
