"""ctypes mirror of include/npgpu.h (the C ABI of the GPU rigid-body step).

Layouts here must match the header field for field; tests check the sizes
against the library's own view (npgpu_abi_version and the struct sizes).
"""
import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libnpgpu.so")

NPGPU_ABI_VERSION = 8

# npgpu_status
OK = 0
ERR_INVALID_HANDLE = 1
ERR_UNSUPPORTED_BODY = 2
ERR_UNSUPPORTED_SHAPE = 3
ERR_NONEMPTY_JOINTS = 4
ERR_NONEMPTY_FORCES = 5
ERR_CAPACITY = 6
ERR_NAN = 7
ERR_TIMEOUT = 8
ERR_CUDA = 9
ERR_INVALID_ARGUMENT = 10

STATUS_NAMES = {
    0: "OK", 1: "INVALID_HANDLE", 2: "UNSUPPORTED_BODY", 3: "UNSUPPORTED_SHAPE", 4: "NONEMPTY_JOINTS",
    5: "NONEMPTY_FORCES", 6: "CAPACITY", 7: "NAN", 8: "TIMEOUT", 9: "CUDA", 10: "INVALID_ARGUMENT",
}

# BodyStatus
BODY_DISABLED, BODY_STATIC, BODY_DYNAMIC, BODY_KINEMATIC = 0, 1, 2, 3
# Body kinds
KIND_RIGID_BODY, KIND_GROUND, KIND_MULTIBODY, KIND_FEM_VOLUME, KIND_FEM_SURFACE, KIND_MASS_SPRING, \
    KIND_MASS_CONSTRAINT = range(7)
# Body flags
BODY_GRAVITY = 1 << 0
BODY_LOCK_TX, BODY_LOCK_TY, BODY_LOCK_TZ = 1 << 1, 1 << 2, 1 << 3
BODY_LOCK_RX, BODY_LOCK_RY, BODY_LOCK_RZ = 1 << 4, 1 << 5, 1 << 6
BODY_CAN_SLEEP = 1 << 7

# npgpu_params.solver_schedule
SCHEDULE_AUTO, SCHEDULE_GRID, SCHEDULE_WORLDS = 0, 1, 2
BODY_LINEAR_INTERP = 1 << 8
# Shapes
SHAPE_BALL, SHAPE_CUBOID, SHAPE_OTHER, SHAPE_CAPSULE = 0, 1, 2, 3
# Combine modes
COMBINE_AVERAGE, COMBINE_MIN, COMBINE_MULTIPLY, COMBINE_MAX = 0, 1, 2, 3

FLT_MAX = float(np.finfo(np.float32).max)


class Handle(C.Structure):
    _fields_ = [("index", C.c_uint64), ("generation", C.c_uint64)]


class BodyDesc(C.Structure):
    _fields_ = [
        ("position", C.c_float * 7),
        ("velocity", C.c_float * 6),
        ("local_inertia", C.c_float * 7),
        ("local_com", C.c_float * 3),
        ("linear_damping", C.c_float),
        ("angular_damping", C.c_float),
        ("max_linear_velocity", C.c_float),
        ("max_angular_velocity", C.c_float),
        ("sleep_threshold", C.c_float),
        ("status", C.c_uint32),
        ("kind", C.c_uint32),
        ("flags", C.c_uint32),
        ("world", C.c_uint32),
    ]


class ColliderDesc(C.Structure):
    _fields_ = [
        ("body", Handle),
        ("position_wrt_body", C.c_float * 7),
        ("shape_params", C.c_float * 3),
        ("margin", C.c_float),
        ("density", C.c_float),
        ("linear_prediction", C.c_float),
        ("angular_prediction", C.c_float),
        ("friction", C.c_float),
        ("restitution", C.c_float),
        ("friction_combine", C.c_uint32),
        ("restitution_combine", C.c_uint32),
        ("shape", C.c_uint32),
        ("is_sensor", C.c_uint32),
        ("ccd_enabled", C.c_uint32),
    ]


# Joint kinds (BallConstraint, FixedConstraint, RevoluteConstraint, CartesianConstraint,
# PlanarConstraint, RectangularConstraint, UniversalConstraint)
(JOINT_BALL, JOINT_FIXED, JOINT_REVOLUTE, JOINT_CARTESIAN, JOINT_PLANAR, JOINT_RECTANGULAR, JOINT_UNIVERSAL,
 JOINT_PRISMATIC, JOINT_CYLINDRICAL, JOINT_PIN_SLOT) = range(10)
JOINT_MIN_OFFSET, JOINT_MAX_OFFSET = 1, 2


class JointDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32),
        ("pad", C.c_uint32),
        ("body1", Handle),
        ("body2", Handle),
        ("anchor1", C.c_float * 3),
        ("anchor2", C.c_float * 3),
        ("frame1", C.c_float * 4),
        ("frame2", C.c_float * 4),
        ("break_force", C.c_float),
        ("break_torque", C.c_float),
        ("axis1", C.c_float * 3),
        ("axis2", C.c_float * 3),
        ("angle", C.c_float),
        ("limit_flags", C.c_uint32),
        ("axis3", C.c_float * 3),
        ("min_offset", C.c_float),
        ("max_offset", C.c_float),
        ("pad2", C.c_uint32),
    ]


class JointState(C.Structure):
    _fields_ = [("impulses", C.c_float * 6), ("limit_impulse", C.c_float), ("broken", C.c_uint32),
                ("active", C.c_uint32), ("pad", C.c_uint32)]


def joint_desc(kind, body1, body2, anchor1=(0, 0, 0), anchor2=(0, 0, 0), frame1=(0, 0, 0, 1), frame2=(0, 0, 0, 1),
               break_force=None, break_torque=None, axis1=(1, 0, 0), axis2=(1, 0, 0), angle=0.0, axis3=(1, 0, 0),
               min_offset=None, max_offset=None):
    """A JointDesc as the joint kind's ::new builds it (body handles as
    (index, generation) pairs or Handle)."""
    d = JointDesc()
    d.kind = kind
    for f, h in (("body1", body1), ("body2", body2)):
        hh = h if isinstance(h, Handle) else Handle(int(h[0]), int(h[1]))
        setattr(d, f, hh)
    d.anchor1[:] = [float(x) for x in anchor1]
    d.anchor2[:] = [float(x) for x in anchor2]
    d.frame1[:] = [float(x) for x in frame1]
    d.frame2[:] = [float(x) for x in frame2]
    d.break_force = FLT_MAX if break_force is None else break_force
    d.break_torque = FLT_MAX if break_torque is None else break_torque
    d.axis1[:] = [float(x) for x in axis1]
    d.axis2[:] = [float(x) for x in axis2]
    d.axis3[:] = [float(x) for x in axis3]
    d.angle = float(angle)
    d.limit_flags = (JOINT_MIN_OFFSET if min_offset is not None else 0) | (JOINT_MAX_OFFSET if max_offset is not None else 0)
    d.min_offset = 0.0 if min_offset is None else float(min_offset)
    d.max_offset = 0.0 if max_offset is None else float(max_offset)
    return d


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_float),
        ("erp", C.c_float),
        ("warmstart_coeff", C.c_float),
        ("restitution_velocity_threshold", C.c_float),
        ("allowed_linear_error", C.c_float),
        ("allowed_angular_error", C.c_float),
        ("max_linear_correction", C.c_float),
        ("max_angular_correction", C.c_float),
        ("max_stabilization_multiplier", C.c_float),
        ("max_velocity_iterations", C.c_uint32),
        ("max_position_iterations", C.c_uint32),
        ("max_ccd_position_iterations", C.c_uint32),
        ("max_ccd_substeps", C.c_uint32),
        ("solve_to_tolerance", C.c_uint32),
        ("residual_tolerance", C.c_float),
        ("max_iterations_to_tolerance", C.c_uint32),
        ("warmstart_mode", C.c_uint32),
        ("broad_phase_margin", C.c_float),
        ("activation_mix", C.c_float),
        ("profile", C.c_uint32),
        ("solver_schedule", C.c_uint32),
        ("use_graph", C.c_uint32),
        ("world_threads", C.c_uint32),
        ("sweep_order", C.c_uint32),
        ("ccd_on_penetration_enabled", C.c_uint32),
    ]


class Counters(C.Structure):
    _fields_ = [
        ("step_time", C.c_double),
        ("collision_detection_time", C.c_double),
        ("broad_phase_time", C.c_double),
        ("narrow_phase_time", C.c_double),
        ("island_construction_time", C.c_double),
        ("solver_time", C.c_double),
        ("assembly_time", C.c_double),
        ("velocity_resolution_time", C.c_double),
        ("velocity_update_time", C.c_double),
        ("position_resolution_time", C.c_double),
        ("colouring_time", C.c_double),
        ("steps", C.c_uint64),
        ("num_pairs", C.c_uint32),
        ("num_manifolds", C.c_uint32),
        ("num_contacts", C.c_uint32),
        ("num_solver_contacts", C.c_uint32),
        ("num_constraints", C.c_uint32),
        ("num_colours", C.c_uint32),
        ("num_active_bodies", C.c_uint32),
        ("velocity_iterations", C.c_uint32),
        ("residual", C.c_double),
        ("residual_initial", C.c_double),
        ("max_penetration", C.c_double),
        ("kinetic_energy", C.c_double),
        ("velocity_task_ms", C.c_double),
        ("velocity_wait_ms", C.c_double),
        ("velocity_kernel_ms", C.c_double),
        ("velocity_tasks", C.c_uint64),
        ("learned_starts", C.c_uint32),
        ("learned_kept", C.c_uint32),
        ("graph_replay", C.c_uint32),
        ("ccd_substeps", C.c_uint32),
        ("ccd_impacts", C.c_uint32),
        ("reserved", C.c_uint32),
        ("ccd_toi_computation_time", C.c_double),
        ("ccd_solver_time", C.c_double),
        ("ccd_broad_phase_time", C.c_double),
        ("ccd_narrow_phase_time", C.c_double),
        ("ccd_world_time_max", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Contact(C.Structure):
    _fields_ = [
        ("collider1", C.c_uint32),
        ("collider2", C.c_uint32),
        ("feature_key", C.c_uint32),
        ("kinematic", C.c_uint32),
        ("world1", C.c_float * 3),
        ("world2", C.c_float * 3),
        ("normal", C.c_float * 3),
        ("depth", C.c_float),
        ("impulse", C.c_float * 3),
        ("colour", C.c_uint32),
    ]


def default_params():
    """IntegrationParameters::default() (src/solver/integration_parameters.rs:169-189)
    plus the GPU-only defaults."""
    p = Params()
    p.dt = 1.0 / 60.0
    p.erp = 0.2
    p.warmstart_coeff = 1.0
    p.restitution_velocity_threshold = 1.0
    p.allowed_linear_error = 0.001
    p.allowed_angular_error = 0.001
    p.max_linear_correction = 0.2
    p.max_angular_correction = 0.2
    p.max_stabilization_multiplier = 0.2
    p.max_velocity_iterations = 8
    p.max_position_iterations = 3
    p.max_ccd_position_iterations = 10
    p.max_ccd_substeps = 1
    p.solve_to_tolerance = 0
    p.residual_tolerance = 1e-4
    p.max_iterations_to_tolerance = 256
    p.warmstart_mode = 0
    p.broad_phase_margin = 0.01
    p.activation_mix = 0.01
    p.profile = 0
    p.solver_schedule = SCHEDULE_AUTO
    p.use_graph = 1
    p.world_threads = 0
    p.sweep_order = SWEEP_SEPARATE
    p.ccd_on_penetration_enabled = 0
    return p


class RayHit(C.Structure):
    _fields_ = [("ray", C.c_uint32), ("collider", C.c_uint32), ("toi", C.c_float), ("normal", C.c_float * 3)]


class ContactEvent(C.Structure):
    _fields_ = [("collider1", C.c_uint32), ("collider2", C.c_uint32), ("stopped", C.c_uint32)]


# ncollide3d query::Proximity of a pair with a sensor.
PROXIMITY_INTERSECTING, PROXIMITY_WITHIN_MARGIN, PROXIMITY_DISJOINT = 0, 1, 2


class ProximityEvent(C.Structure):
    _fields_ = [("collider1", C.c_uint32), ("collider2", C.c_uint32), ("prev_status", C.c_uint32),
                ("new_status", C.c_uint32)]


ALL_WORLDS = 0xffffffff


def contacts_to_numpy(arr, n):
    """Converts a ctypes Contact array into a dict of numpy arrays."""
    raw = np.ctypeslib.as_array(arr, shape=(n,)) if n else None
    if n == 0:
        z = np.zeros((0,), np.uint32)
        return {"collider1": z, "collider2": z, "feature_key": z, "kinematic": z,
                "world1": np.zeros((0, 3), np.float32), "world2": np.zeros((0, 3), np.float32),
                "normal": np.zeros((0, 3), np.float32), "depth": np.zeros((0,), np.float32),
                "impulse": np.zeros((0, 3), np.float32), "colour": z}
    return {k: np.array(raw[k]) for k in raw.dtype.names}


def load_library(path=LIB_PATH):
    """Loads libnpgpu.so and declares every entry point of include/npgpu.h."""
    if not os.path.exists(path):
        raise RuntimeError(f"libnpgpu.so is not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    P = C.POINTER
    W = C.c_void_p
    decl = {
        "npgpu_abi_version": (C.c_uint32, []),
        "npgpu_default_params": (None, [P(Params)]),
        "npgpu_create": (W, [P(Params), P(C.c_float), C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_int)]),
        "npgpu_destroy": (None, [W]),
        "npgpu_stream": (C.c_void_p, [W]),
        "npgpu_set_params": (C.c_int, [W, P(Params)]),
        "npgpu_set_gravity": (C.c_int, [W, P(C.c_float)]),
        "npgpu_upsert_bodies": (C.c_int, [W, C.c_uint32, P(Handle), P(BodyDesc)]),
        "npgpu_upsert_colliders": (C.c_int, [W, C.c_uint32, P(Handle), P(ColliderDesc)]),
        "npgpu_remove_bodies": (C.c_int, [W, C.c_uint32, P(Handle)]),
        "npgpu_remove_colliders": (C.c_int, [W, C.c_uint32, P(Handle)]),
        "npgpu_apply_forces": (C.c_int, [W, C.c_uint32, P(Handle), P(C.c_float), C.c_int]),
        "npgpu_upsert_joints": (C.c_int, [W, C.c_uint32, P(Handle), P(JointDesc)]),
        "npgpu_remove_joints": (C.c_int, [W, C.c_uint32, P(Handle)]),
        "npgpu_get_joints": (C.c_int, [W, C.c_uint32, P(Handle), P(JointState)]),
        "npgpu_step": (C.c_int, [W, C.c_uint32, C.c_uint32, C.c_uint32]),
        "npgpu_synchronize": (C.c_int, [W]),
        "npgpu_download_bodies": (C.c_int, [W, C.c_uint32, C.c_uint32, P(C.c_float), P(C.c_float),
                                            P(C.c_float), P(C.c_uint8)]),
        "npgpu_download_mass_properties": (C.c_int, [W, C.c_uint32, C.c_uint32, P(C.c_float), P(C.c_float)]),
        "npgpu_get_pairs": (C.c_int, [W, P(C.c_uint32), C.c_uint32, P(C.c_uint32)]),
        "npgpu_get_aabbs": (C.c_int, [W, C.c_uint32, C.c_uint32, P(C.c_float)]),
        "npgpu_get_contacts": (C.c_int, [W, P(Contact), C.c_uint32, P(C.c_uint32)]),
        "npgpu_get_counters": (C.c_int, [W, P(Counters)]),
        "npgpu_last_error": (C.c_char_p, [W]),
        "npgpu_find_pairs_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                              C.c_void_p, C.c_void_p]),
        "npgpu_autotune": (C.c_int, [W, C.c_uint32, P(C.c_uint32), P(C.c_uint32), P(C.c_float)]),
        "npgpu_interferences_with_rays": (C.c_int, [W, C.c_uint32, P(C.c_float), P(C.c_float), C.c_uint32,
                                                    P(RayHit), C.c_uint32, P(C.c_uint32)]),
        "npgpu_interferences_with_points": (C.c_int, [W, C.c_uint32, P(C.c_float), C.c_uint32, P(C.c_uint32),
                                                      C.c_uint32, P(C.c_uint32)]),
        "npgpu_interferences_with_aabbs": (C.c_int, [W, C.c_uint32, P(C.c_float), C.c_uint32, P(C.c_uint32),
                                                     C.c_uint32, P(C.c_uint32)]),
        "npgpu_enable_contact_events": (C.c_int, [W, C.c_uint32]),
        "npgpu_contact_events": (C.c_int, [W, P(ContactEvent), C.c_uint32, P(C.c_uint32)]),
        "npgpu_proximity_events": (C.c_int, [W, P(ProximityEvent), C.c_uint32, P(C.c_uint32)]),
        "npgpu_mlp_set": (C.c_int, [W, P(C.c_float), C.c_uint32]),
        "npgpu_mlp_get": (C.c_int, [W, P(C.c_float), C.c_uint32]),
        "npgpu_mlp_record": (C.c_int, [W, C.c_uint32]),
        "npgpu_mlp_samples": (C.c_int, [W, P(C.c_float), C.c_uint32, P(C.c_uint32)]),
        "npgpu_mlp_load_samples": (C.c_int, [W, P(C.c_float), C.c_uint32]),
        "npgpu_mlp_train": (C.c_int, [W, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, C.c_uint32,
                                      P(C.c_float)]),
        "npgpu_mlp_grad": (C.c_int, [W, P(C.c_float), C.c_uint32, P(C.c_float), P(C.c_float)]),
    }
    for name, (res, args) in decl.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


# Every entry point include/npgpu.h declares (checked by the CPU tests).
EXPORTED = [
    "npgpu_abi_version", "npgpu_default_params", "npgpu_create", "npgpu_destroy", "npgpu_stream",
    "npgpu_set_params", "npgpu_set_gravity", "npgpu_upsert_bodies", "npgpu_upsert_colliders",
    "npgpu_remove_bodies", "npgpu_remove_colliders", "npgpu_apply_forces", "npgpu_upsert_joints",
    "npgpu_remove_joints", "npgpu_get_joints", "npgpu_step",
    "npgpu_synchronize", "npgpu_download_bodies", "npgpu_download_mass_properties", "npgpu_get_pairs",
    "npgpu_get_aabbs", "npgpu_get_contacts", "npgpu_get_counters", "npgpu_last_error", "npgpu_find_pairs_static",
    "npgpu_interferences_with_rays", "npgpu_interferences_with_points", "npgpu_interferences_with_aabbs",
    "npgpu_enable_contact_events", "npgpu_contact_events", "npgpu_proximity_events",
    "npgpu_autotune", "npgpu_mlp_set", "npgpu_mlp_get", "npgpu_mlp_record", "npgpu_mlp_samples", "npgpu_mlp_load_samples", "npgpu_mlp_train", "npgpu_mlp_grad",
]

# Learned warm start (npgpu_mlp_*).
WARMSTART_CACHE, WARMSTART_NONE, WARMSTART_LEARNED, WARMSTART_LEARNED_ALL = 0, 1, 2, 3
SWEEP_SEPARATE, SWEEP_MANIFOLD = 0, 1
MLP_IN, MLP_HIDDEN, MLP_OUT = 24, 64, 3
MLP_PARAMS = 6009
MLP_TRAINABLE = 5955
MLP_SAMPLE_FLOATS = 28
MLP_INIT = 1
