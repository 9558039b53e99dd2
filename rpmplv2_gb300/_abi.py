"""ctypes mirror of include/rpm_gpu.h (structs and constants only)."""
import ctypes

RPM_MAX_DOF = 32

RPM_OK = 0
RPM_ERR_INVALID = -1
RPM_ERR_CUDA = -2
RPM_ERR_NOMEM = -3
RPM_ERR_TIMEOUT = -4
RPM_ERR_ADMISSION = -5
RPM_ERR_RANGE = -6

RPM_ROBOT_CHAIN = 0
RPM_ROBOT_XARM6 = 1
RPM_ROBOT_SPATIAL = 2

RPM_OBS_GROUND = 0x1
RPM_OBS_DYNAMIC = 0x2

RPM_PREC_FP64 = 0
RPM_PREC_FP32_RECHECK = 1
RPM_PREC_FP32_REF = 2

PRECISIONS = {"fp64": RPM_PREC_FP64, "fp32_recheck": RPM_PREC_FP32_RECHECK, "fp32_ref": RPM_PREC_FP32_REF}

RPM_LAYOUT_AUTO = 0
RPM_LAYOUT_LANE = 1
RPM_LAYOUT_WARP = 2

LAYOUTS = {"auto": RPM_LAYOUT_AUTO, "lane": RPM_LAYOUT_LANE, "warp": RPM_LAYOUT_WARP}


class RobotDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("num_dofs", ctypes.c_int32),
        ("ground_included", ctypes.c_int32),
        ("gripper_length", ctypes.c_float),
        ("joint_axis", ctypes.c_int32 * RPM_MAX_DOF),
        ("origin_xyz", (ctypes.c_double * 3) * (RPM_MAX_DOF + 1)),
        ("origin_rot", (ctypes.c_double * 9) * (RPM_MAX_DOF + 1)),
        ("capsule_radius", ctypes.c_float * RPM_MAX_DOF),
        ("limits", (ctypes.c_float * 2) * RPM_MAX_DOF),
    ]


class Params(ctypes.Structure):
    _fields_ = [("equality_threshold", ctypes.c_double), ("max_distance", ctypes.c_double)]


class TileShape(ctypes.Structure):
    """rpm_tile_shape."""
    _fields_ = [
        ("layout", ctypes.c_int32),
        ("configs_per_warp", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("ms", ctypes.c_float),
    ]

    def as_dict(self):
        return {"layout": {1: "lane", 2: "warp"}.get(self.layout, "auto"), "configs_per_warp": self.configs_per_warp,
                "ctas_per_sm": self.ctas_per_sm, "ms": self.ms}


RPM_OUT_VALID, RPM_OUT_DIST, RPM_OUT_PROFILE = 1, 2, 4


class CheckStats(ctypes.Structure):
    _fields_ = [
        ("configs", ctypes.c_int64),
        ("rechecked", ctypes.c_int64),
        ("overflow", ctypes.c_int64),
        ("device_status", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class BatchItem(ctypes.Structure):
    _fields_ = [
        ("scene_id", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("q_dev", ctypes.c_void_p),
        ("num_configs", ctypes.c_int64),
        ("valid_dev", ctypes.c_void_p),
        ("dist_dev", ctypes.c_void_p),
        ("profile_dev", ctypes.c_void_p),
    ]


class EdgeBatchItem(ctypes.Structure):
    """rpm_edge_batch_item."""
    _fields_ = [
        ("scene_id", ctypes.c_int32),
        ("num_checks", ctypes.c_int32),
        ("num_edges", ctypes.c_int64),
        ("q1_dev", ctypes.c_void_p),
        ("q2_dev", ctypes.c_void_p),
        ("step", ctypes.c_float),
        ("valid_dev", ctypes.c_void_p),
        ("checks_dev", ctypes.c_void_p),
    ]


class SpineParams(ctypes.Structure):
    """rpm_spine_params."""
    _fields_ = [
        ("num_layers", ctypes.c_int32),
        ("num_iter", ctypes.c_int32),
        ("expanded", ctypes.c_int32),
        ("d_crit", ctypes.c_float),
    ]


class MovingBox(ctypes.Structure):
    """rpm_moving_box."""
    _fields_ = [
        ("index", ctypes.c_int32),
        ("max_vel", ctypes.c_float),
        ("dim", ctypes.c_float * 3),
        ("pos", ctypes.c_float * 3),
        ("quat_xyzw", ctypes.c_float * 4),
    ]


class ScenarioInfo(ctypes.Structure):
    """rpm_scenario_info."""
    _fields_ = [
        ("type", ctypes.c_char * 32),
        ("num_dofs", ctypes.c_int32),
        ("ground_included", ctypes.c_int32),
        ("num_radii", ctypes.c_int32),
        ("num_obstacles", ctypes.c_int32),
        ("capsules_radius", ctypes.c_float * RPM_MAX_DOF),
        ("gripper_length", ctypes.c_float),
        ("ws_center", ctypes.c_float * 3),
        ("ws_radius", ctypes.c_float),
        ("q_start", ctypes.c_float * RPM_MAX_DOF),
        ("q_goal", ctypes.c_float * RPM_MAX_DOF),
    ]
