"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this module, and only as the checker or as the timed CPU reference.
"""
import ctypes as C
import os

import numpy as np

from nphysics_gb300 import abi

from . import build_oracle

ORDER_REFERENCE = 0
ORDER_COLOUR = 1

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.POINTER
        W = C.c_void_p
        decl = {
            "orc_create": (W, [C.c_int, P(abi.Params), P(C.c_float)]),
            "orc_destroy": (None, [W]),
            "orc_set_order": (None, [W, C.c_int]),
            "orc_mlp_set": (None, [W, C.POINTER(C.c_float), C.c_uint32]),
            "orc_set_params": (None, [W, P(abi.Params)]),
            "orc_upsert_bodies": (C.c_int, [W, C.c_uint32, C.c_void_p, C.c_void_p]),
            "orc_upsert_colliders": (C.c_int, [W, C.c_uint32, C.c_void_p, C.c_void_p]),
            "orc_remove_bodies": (C.c_int, [W, C.c_uint32, C.c_void_p]),
            "orc_remove_colliders": (C.c_int, [W, C.c_uint32, C.c_void_p]),
            "orc_apply_forces": (C.c_int, [W, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int]),
            "orc_upsert_joints": (C.c_int, [W, C.c_uint32, C.c_void_p, C.c_void_p]),
            "orc_remove_joints": (C.c_int, [W, C.c_uint32, C.c_void_p]),
            "orc_get_joints": (C.c_int, [W, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
            "orc_step": (C.c_int, [W, C.c_uint32]),
            "orc_collision_detection": (None, [W]),
            "orc_download_bodies": (C.c_int, [W, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p]),
            "orc_download_mass_properties": (C.c_int, [W, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
            "orc_set_body_state": (C.c_int, [W, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
            "orc_get_pairs": (C.c_uint32, [W, C.c_void_p, C.c_uint32]),
            "orc_brute_force_pairs": (C.c_uint32, [W, C.c_void_p, C.c_uint32]),
            "orc_get_aabbs": (C.c_int, [W, C.c_uint32, C.c_uint32, C.c_void_p]),
            "orc_get_contacts": (C.c_uint32, [W, C.c_void_p, C.c_uint32]),
            "orc_get_contacts_f64": (C.c_uint32, [W, C.c_void_p, C.c_uint32]),
            "orc_get_counters": (None, [W, P(abi.Counters)]),
            "orc_collider_distance": (C.c_double, [W, C.c_uint32, C.c_uint32, P(C.c_double * 3)]),
            "orc_pair_toi": (C.c_int, [W, C.c_uint32, C.c_uint32, C.c_double, P(C.c_double)]),
            "orc_last_error": (C.c_char_p, [W]),
            "orc_record_events": (None, [W, C.c_int]),
            "orc_contact_events": (C.c_uint32, [W, C.c_void_p, C.c_uint32]),
            "orc_proximity_events": (C.c_uint32, [W, C.c_void_p, C.c_uint32]),
            "orc_rays": (C.c_uint32, [W, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
            "orc_overlaps": (C.c_uint32, [W, C.c_int, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
        }
        for name, (res, args) in decl.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class OracleWorld:
    """The oracle with the same surface as nphysics_gb300.GpuWorld."""

    def __init__(self, params=None, gravity=(0.0, -9.81, 0.0), precision=32, order=ORDER_REFERENCE):
        self.L = lib()
        self.params = params if params is not None else abi.default_params()
        g = (C.c_float * 3)(*gravity)
        self.w = self.L.orc_create(precision, C.byref(self.params), g)
        self.L.orc_set_order(self.w, order)
        self.num_bodies = 0
        self.num_colliders = 0

    def close(self):
        if self.w:
            self.L.orc_destroy(self.w)
            self.w = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s, what):
        if s != 0:
            raise RuntimeError(f"oracle {what}: {abi.STATUS_NAMES.get(s, s)}: "
                               f"{self.L.orc_last_error(self.w).decode()}")

    def set_order(self, order):
        self.L.orc_set_order(self.w, order)

    def mlp_set(self, params):
        """The learned warm start's network (the fp32 layout of npgpu_mlp_set)."""
        params = np.ascontiguousarray(params, np.float32)
        self.L.orc_mlp_set(self.w, params.ctypes.data_as(C.POINTER(C.c_float)), params.size)

    def set_params(self, params):
        self.params = params
        self.L.orc_set_params(self.w, C.byref(params))

    def load_scene(self, scene):
        b = np.ascontiguousarray(scene.bodies)
        c = np.ascontiguousarray(scene.colliders)
        self._check(self.L.orc_upsert_bodies(self.w, len(b), _ptr(scene.body_handles), _ptr(b)), "upsert bodies")
        self._check(self.L.orc_upsert_colliders(self.w, len(c), _ptr(scene.collider_handles), _ptr(c)),
                    "upsert colliders")
        self.num_bodies = max(self.num_bodies, len(b))
        self.num_colliders = max(self.num_colliders, len(c))
        if len(getattr(scene, "joints", ())):
            self.upsert_joints(scene.joint_handles, scene.joints)

    def upsert_joints(self, handles, descs):
        d = np.ascontiguousarray(descs)
        self._check(self.L.orc_upsert_joints(self.w, len(d), _ptr(np.ascontiguousarray(handles)), _ptr(d)),
                    "upsert joints")

    def remove_joints(self, handles):
        self._check(self.L.orc_remove_joints(self.w, len(handles), _ptr(np.ascontiguousarray(handles))),
                    "remove joints")

    def joints(self, handles):
        """(impulses (n, 7) f64: linear, angular, the limit's; broken (n,), active (n,)) after the last step."""
        h = np.ascontiguousarray(handles)
        imp = np.zeros((len(h), 7), np.float64)
        flags = np.zeros((len(h), 2), np.uint32)
        self._check(self.L.orc_get_joints(self.w, len(h), _ptr(h), _ptr(imp), _ptr(flags)), "get joints")
        return imp, flags[:, 0].astype(bool), flags[:, 1].astype(bool)

    def upsert_bodies(self, handles, descs):
        self._check(self.L.orc_upsert_bodies(self.w, len(descs), _ptr(handles), _ptr(descs)), "upsert bodies")
        self.num_bodies = max(self.num_bodies, int(handles["index"].max()) + 1)

    def upsert_colliders(self, handles, descs):
        self._check(self.L.orc_upsert_colliders(self.w, len(descs), _ptr(handles), _ptr(descs)), "upsert colliders")
        self.num_colliders = max(self.num_colliders, int(handles["index"].max()) + 1)

    def remove_bodies(self, handles):
        self._check(self.L.orc_remove_bodies(self.w, len(handles), _ptr(handles)), "remove bodies")

    def remove_colliders(self, handles):
        self._check(self.L.orc_remove_colliders(self.w, len(handles), _ptr(handles)), "remove colliders")

    def apply_forces(self, handles, forces, wake=True):
        f = np.ascontiguousarray(forces, np.float32)
        self._check(self.L.orc_apply_forces(self.w, len(handles), _ptr(handles), _ptr(f), int(wake)), "apply forces")

    def step(self, n=1):
        self._check(self.L.orc_step(self.w, n), "step")

    def collision_detection(self):
        self.L.orc_collision_detection(self.w)

    def set_body_state(self, first, pos=None, vel=None):
        n = len(pos) if pos is not None else len(vel)
        p = np.ascontiguousarray(pos, np.float32) if pos is not None else None
        v = np.ascontiguousarray(vel, np.float32) if vel is not None else None
        self._check(self.L.orc_set_body_state(self.w, first, n, _ptr(p), _ptr(v)), "set body state")

    def bodies(self, first=0, n=None):
        n = self.num_bodies - first if n is None else n
        pos = np.zeros((n, 7), np.float64)
        vel = np.zeros((n, 6), np.float64)
        energy = np.zeros(n, np.float64)
        active = np.zeros(n, np.uint8)
        self._check(self.L.orc_download_bodies(self.w, first, n, _ptr(pos), _ptr(vel), _ptr(energy), _ptr(active)),
                    "download bodies")
        return {"position": pos, "velocity": vel, "energy": energy, "active": active}

    def mass_properties(self, first=0, n=None):
        n = self.num_bodies - first if n is None else n
        inertia = np.zeros((n, 7), np.float64)
        com = np.zeros((n, 3), np.float64)
        self._check(self.L.orc_download_mass_properties(self.w, first, n, _ptr(inertia), _ptr(com)), "mass props")
        return inertia, com

    def pairs(self):
        n = self.L.orc_get_pairs(self.w, None, 0)
        out = np.zeros((max(n, 1), 2), np.uint32)
        self.L.orc_get_pairs(self.w, _ptr(out), n)
        return out[:n]

    def brute_force_pairs(self):
        n = self.L.orc_brute_force_pairs(self.w, None, 0)
        out = np.zeros((max(n, 1), 2), np.uint32)
        self.L.orc_brute_force_pairs(self.w, _ptr(out), n)
        return out[:n]

    def aabbs(self, first=0, n=None):
        n = self.num_colliders - first if n is None else n
        out = np.zeros((n, 6), np.float64)
        self._check(self.L.orc_get_aabbs(self.w, first, n, _ptr(out)), "aabbs")
        return out

    def contacts(self):
        n = self.L.orc_get_contacts(self.w, None, 0)
        arr = (abi.Contact * max(n, 1))()
        self.L.orc_get_contacts(self.w, C.cast(arr, C.c_void_p), n)
        return abi.contacts_to_numpy(arr, n)

    def contacts_f64(self):
        n = self.L.orc_get_contacts_f64(self.w, None, 0)
        out = np.zeros((max(n, 1), 13), np.float64)
        self.L.orc_get_contacts_f64(self.w, _ptr(out), n)
        return out[:n]

    def collider_distance(self, c1, c2):
        """Distance of two colliders' shapes at the current poses, and the
        unit direction from the first toward the second."""
        d = (C.c_double * 3)()
        dist = self.L.orc_collider_distance(self.w, c1, c2, C.byref(d))
        return dist, np.array(d[:])

    def pair_toi(self, c1, c2, horizon):
        """Time of impact of two colliders moving at their bodies' velocities
        from the current poses: (status, toi), status -1 none, 0 an impact,
        1 overlapping at the start."""
        t = C.c_double(0.0)
        r = self.L.orc_pair_toi(self.w, c1, c2, horizon, C.byref(t))
        return r, t.value

    def counters(self):
        c = abi.Counters()
        self.L.orc_get_counters(self.w, C.byref(c))
        return c.as_dict()

    # ---- contact events and geometric queries (same surface as GpuWorld) ----
    def enable_contact_events(self, capacity=1 << 20):
        self.L.orc_record_events(self.w, 1 if capacity else 0)

    def contact_events(self):
        """(collider1, collider2, stopped) rows, sorted."""
        n = self.L.orc_contact_events(self.w, None, 0)
        out = np.zeros((max(n, 1), 3), np.uint32)
        self.L.orc_contact_events(self.w, _ptr(out), n)
        out = out[:n]
        return out[np.lexsort((out[:, 2], out[:, 1], out[:, 0]))] if n else out

    def proximity_events(self):
        """(collider1, collider2, previous, new) rows by pair, each pair's in
        pass order."""
        n = self.L.orc_proximity_events(self.w, None, 0)
        out = np.zeros((max(n, 1), 4), np.uint32)
        self.L.orc_proximity_events(self.w, _ptr(out), n)
        out = out[:n]
        return out[np.lexsort((out[:, 1], out[:, 0]))] if n else out

    def rays(self, rays6, max_toi, world=0xffffffff):
        rays6 = np.ascontiguousarray(rays6, np.float32).reshape(-1, 6)
        max_toi = np.ascontiguousarray(max_toi, np.float32).reshape(-1)
        n = self.L.orc_rays(self.w, len(rays6), _ptr(rays6), _ptr(max_toi), world, None, 0)
        out = np.zeros((max(n, 1), 6), np.float64)
        self.L.orc_rays(self.w, len(rays6), _ptr(rays6), _ptr(max_toi), world, _ptr(out), n)
        return out[:n]

    def overlaps(self, kind, q, world=0xffffffff):
        q = np.ascontiguousarray(q, np.float32)
        nq = len(q)
        n = self.L.orc_overlaps(self.w, kind, nq, _ptr(q), world, None, 0)
        out = np.zeros((max(n, 1), 2), np.uint32)
        self.L.orc_overlaps(self.w, kind, nq, _ptr(q), world, _ptr(out), n)
        return out[:n]

    def points(self, points3, world=0xffffffff):
        return self.overlaps(1, np.ascontiguousarray(points3, np.float32).reshape(-1, 3), world)

    def aabb_query(self, aabbs6, world=0xffffffff):
        return self.overlaps(2, np.ascontiguousarray(aabbs6, np.float32).reshape(-1, 6), world)
