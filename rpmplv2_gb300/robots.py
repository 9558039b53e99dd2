"""Robot models of the reference as kinematic descriptors.

The tables are transcribed from the reference's URDFs (kdl_parser builds a
chain of segments, each a fixed origin followed by a revolute joint):

* planar_2dof   data/planar_2dof/planar_2dof.urdf   (robots::Planar2DOF, src/robots/Planar2DOF.cpp)
* planar_10dof  data/planar_10dof/planar_10dof.urdf (robots::Planar10DOF)
* spatial_Ndof  data/spatial_{10,14,18,22}dof/*.urdf (robots::Spatial10DOF family, src/robots/Spatial10DOF.cpp:5-9)
* xarm6         data/xarm6/xarm6.urdf               (robots::xArm6, src/robots/xArm6.cpp)

Default capsule radius of the Planar2DOF family is the URDF link box's
dim.y / 2 = 0.025 (Planar2DOF.cpp:51); scenarios override it
(src/scenario/Scenario.cpp:36-51).  Joint-origin rotations follow URDF rpy ->
quaternion -> rotation matrix, with the rpy values exactly as written
(e.g. -1.5708, not -pi/2).
"""
import math

import numpy as np

from ._abi import RobotDesc, RPM_MAX_DOF, RPM_ROBOT_CHAIN, RPM_ROBOT_SPATIAL, RPM_ROBOT_XARM6

PI_URDF = 3.14159

SPATIAL_LINK_OFFSET = {10: 0.1, 14: 0.0692, 18: 0.05294, 22: 0.042857}

XARM6_JOINTS = [  # (xyz, rpy, (lower, upper)) of joint1..joint6 (xarm6.urdf)
    ((0.0, 0.0, 0.267), (0.0, 0.0, 0.0), (-3.14159265359, 3.14159265359)),
    ((0.0, 0.0, 0.0), (-1.5708, 0.0, 0.0), (-2.059, 2.0944)),
    ((0.0535, -0.2845, 0.0), (0.0, 0.0, 0.0), (-3.927, 0.19198)),
    ((0.0775, 0.3425, 0.0), (-1.5708, 0.0, 0.0), (-3.14159265359, 3.14159265359)),
    ((0.0, 0.0, 0.0), (1.5708, 0.0, 0.0), (-1.69297, 3.14159265359)),
    ((0.076, 0.097, 0.0), (-1.5708, 0.0, 0.0), (-3.14159265359, 3.14159265359)),
]


def rpy_to_matrix(roll, pitch, yaw):
    """URDF rpy -> unit quaternion (fixed-axis x-y-z) -> row-major 3x3 rotation."""
    phi, the, psi = roll / 2.0, pitch / 2.0, yaw / 2.0
    sphi, cphi = math.sin(phi), math.cos(phi)
    sthe, cthe = math.sin(the), math.cos(the)
    spsi, cpsi = math.sin(psi), math.cos(psi)
    x = sphi * cthe * cpsi - cphi * sthe * spsi
    y = cphi * sthe * cpsi + sphi * cthe * spsi
    z = cphi * cthe * spsi - sphi * sthe * cpsi
    w = cphi * cthe * cpsi + sphi * sthe * spsi
    n = math.sqrt(x * x + y * y + z * z + w * w)
    x, y, z, w = x / n, y / n, z / n, w / n
    x2, y2, z2, w2 = x * x, y * y, z * z, w * w
    return [w2 + x2 - y2 - z2, 2 * x * y - 2 * w * z, 2 * x * z + 2 * w * y,
            2 * x * y + 2 * w * z, w2 - x2 + y2 - z2, 2 * y * z - 2 * w * x,
            2 * x * z - 2 * w * y, 2 * y * z + 2 * w * x, w2 - x2 - y2 + z2]


IDENTITY = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]


class Robot:
    """Host-side robot model: a RobotDesc plus convenience accessors."""

    def __init__(self, name, kind, origins, rots, axes, tool_xyz, radius, limits, ground_included=0,
                 gripper_length=0.0):
        d = len(axes)
        if not (1 <= d <= RPM_MAX_DOF):
            raise ValueError("num_dofs out of range")
        self.name = name
        self.desc = RobotDesc()
        self.desc.kind = kind
        self.desc.num_dofs = d
        self.desc.ground_included = int(ground_included)
        self.desc.gripper_length = float(gripper_length)
        for k in range(d):
            self.desc.joint_axis[k] = int(axes[k])
            for i in range(3):
                self.desc.origin_xyz[k][i] = float(origins[k][i])
            for i in range(9):
                self.desc.origin_rot[k][i] = float(rots[k][i])
            self.desc.limits[k][0] = float(limits[k][0])
            self.desc.limits[k][1] = float(limits[k][1])
        for i in range(3):
            self.desc.origin_xyz[d][i] = float(tool_xyz[i])
        for i in range(9):
            self.desc.origin_rot[d][i] = IDENTITY[i]
        self.set_capsule_radius(radius)

    @property
    def num_dofs(self):
        return self.desc.num_dofs

    @property
    def num_links(self):
        return self.desc.num_dofs

    def set_capsule_radius(self, radius):
        """AbstractRobot::setCapsulesRadius: one value broadcast, or one per link."""
        r = np.atleast_1d(np.asarray(radius, dtype=np.float32))
        if r.size == 1:
            r = np.full(self.num_dofs, r[0], dtype=np.float32)
        if r.size != self.num_dofs:
            raise ValueError("capsule radius count must be 1 or num_dofs")
        for i in range(self.num_dofs):
            self.desc.capsule_radius[i] = float(r[i])

    @property
    def capsule_radius(self):
        return np.array([self.desc.capsule_radius[i] for i in range(self.num_dofs)], dtype=np.float32)

    @property
    def limits(self):
        return np.array([[self.desc.limits[i][0], self.desc.limits[i][1]] for i in range(self.num_dofs)],
                        dtype=np.float32)

    def set_ground_included(self, n):
        self.desc.ground_included = int(n)

    # ---- host FK in float64 (scene generation; not the hot path) ----
    def skeleton_np(self, q):
        """Skeleton points (L+1, 3) in float64 for one configuration."""
        d = self.desc
        D = d.num_dofs
        R = np.eye(3)
        p = np.zeros(3)
        frames = []
        for k in range(D):
            o = np.array(d.origin_xyz[k][:])
            M = np.array(d.origin_rot[k][:]).reshape(3, 3)
            p = R @ o + p
            R = R @ M
            c, s = math.cos(float(q[k])), math.sin(float(q[k]))
            ax = d.joint_axis[k]
            if ax == 0:
                J = np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
            elif ax == 1:
                J = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
            else:
                J = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])
            R = R @ J
            frames.append((R.copy(), p.copy()))
        if d.kind != RPM_ROBOT_XARM6:
            pts = [f[1] for f in frames]
            pts.append(frames[-1][0] @ np.array(d.origin_xyz[D][:]) + frames[-1][1])
            return np.array(pts)
        g = float(d.gripper_length)
        F = frames
        p5 = F[5][1] + g * F[5][0][:, 2]
        return np.array([np.zeros(3), F[1][1], F[2][1], F[3][1] - 0.25 * F[3][0][:, 2], F[4][1],
                         F[4][1] + 0.076 * F[4][0][:, 0], p5 - 0.3 * g * F[5][0][:, 2]])


def planar_2dof(radius=0.025):
    lim = [(-PI_URDF, PI_URDF)] * 2
    return Robot("planar_2dof", RPM_ROBOT_CHAIN, [(0, 0, 0), (1, 0, 0)], [IDENTITY] * 2, [2, 2], (1, 0, 0),
                 radius, lim)


def planar_10dof(radius=0.025):
    origins = [(0, 0, 0)] + [(0.2, 0, 0)] * 9
    return Robot("planar_10dof", RPM_ROBOT_CHAIN, origins, [IDENTITY] * 10, [2] * 10, (0.2, 0, 0), radius,
                 [(-PI_URDF, PI_URDF)] * 10)


def spatial(dofs, radius=0.025, ground_included=0):
    if dofs not in SPATIAL_LINK_OFFSET:
        raise ValueError("spatial robots exist for 10, 14, 18, 22 DOF")
    h = SPATIAL_LINK_OFFSET[dofs]
    origins = [(0, 0, 0), (0, 0, 0.1)] + [(0, 0, h)] * (dofs - 2)
    axes = [2] + [0] * (dofs - 1)
    return Robot("spatial_%ddof" % dofs, RPM_ROBOT_SPATIAL, origins, [IDENTITY] * dofs, axes, (0, 0, h), radius,
                 [(-PI_URDF, PI_URDF)] * dofs, ground_included=ground_included)


def xarm6(radius=(0.047, 0.12, 0.11, 0.09, 0.05, 0.05), gripper_length=0.17, ground_included=2):
    """Defaults are data/xarm6/scenario1/scenario1.yaml:27-33."""
    origins = [j[0] for j in XARM6_JOINTS]
    rots = [rpy_to_matrix(*j[1]) for j in XARM6_JOINTS]
    lim = [j[2] for j in XARM6_JOINTS]
    return Robot("xarm6", RPM_ROBOT_XARM6, origins, rots, [2] * 6, (0, 0, 0), radius, lim,
                 ground_included=ground_included, gripper_length=gripper_length)


def by_name(name, **kw):
    if name == "planar_2dof":
        return planar_2dof(**kw)
    if name == "planar_10dof":
        return planar_10dof(**kw)
    if name == "xarm6":
        return xarm6(**kw)
    if name.startswith("spatial_") and name.endswith("dof"):
        return spatial(int(name[len("spatial_"):-3]), **kw)
    raise ValueError("unknown robot %r" % name)
