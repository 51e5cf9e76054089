"""ctypes binding of libnpgpu.so: the GPU mechanical world as seen from Python.

`GpuWorld` exposes the C ABI of include/npgpu.h one call per entry point. It
is what the tests, the smoke check and the benchmark drive. There is no CPU
fallback: constructing a world without the built library or without a CUDA
device raises.
"""
import ctypes as C

import numpy as np

from . import abi

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = abi.load_library()
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


class NpgpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class GpuWorld:
    def __init__(self, params=None, gravity=(0.0, -9.81, 0.0), capacity_bodies=1024, capacity_colliders=1024,
                 capacity_pairs=None):
        self.L = lib()
        self.params = params if params is not None else abi.default_params()
        g = (C.c_float * 3)(*gravity)
        st = C.c_int(0)
        cap_p = capacity_pairs if capacity_pairs is not None else max(1024, 16 * capacity_colliders)
        self.w = self.L.npgpu_create(C.byref(self.params), g, capacity_bodies, capacity_colliders, cap_p,
                                     C.byref(st))
        if not self.w:
            raise NpgpuError(st.value, self.L.npgpu_last_error(None).decode())
        self.num_bodies = 0
        self.num_colliders = 0
        self._joints = {}                # joint slot -> generation of the joints uploaded

    @classmethod
    def for_scene(cls, scene, params=None, pairs_per_collider=16):
        p = params if params is not None else scene.params()
        w = cls(p, scene.gravity, capacity_bodies=len(scene.bodies), capacity_colliders=len(scene.colliders),
                capacity_pairs=max(1024, pairs_per_collider * len(scene.colliders)) + len(getattr(scene, "joints", ())))
        w.load_scene(scene)
        return w

    def close(self):
        if getattr(self, "w", None):
            self.L.npgpu_destroy(self.w)
            self.w = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s, what=""):
        if s != abi.OK:
            raise NpgpuError(s, f"{what}: {self.L.npgpu_last_error(self.w).decode()}")

    @property
    def stream(self):
        return self.L.npgpu_stream(self.w)

    def set_params(self, params):
        self.params = params
        self._check(self.L.npgpu_set_params(self.w, C.byref(params)), "set_params")

    def set_gravity(self, g):
        self._check(self.L.npgpu_set_gravity(self.w, (C.c_float * 3)(*g)), "set_gravity")

    def upsert_bodies(self, handles, descs):
        descs = np.ascontiguousarray(descs)
        handles = np.ascontiguousarray(handles)
        self._check(self.L.npgpu_upsert_bodies(self.w, len(descs), _ptr(handles, abi.Handle), _ptr(descs, abi.BodyDesc)),
                    "upsert_bodies")
        if len(handles):
            self.num_bodies = max(self.num_bodies, int(handles["index"].max()) + 1)

    def upsert_colliders(self, handles, descs):
        descs = np.ascontiguousarray(descs)
        handles = np.ascontiguousarray(handles)
        self._check(self.L.npgpu_upsert_colliders(self.w, len(descs), _ptr(handles, abi.Handle),
                                                  _ptr(descs, abi.ColliderDesc)), "upsert_colliders")
        if len(handles):
            self.num_colliders = max(self.num_colliders, int(handles["index"].max()) + 1)

    def load_scene(self, scene):
        self.upsert_bodies(scene.body_handles, scene.bodies)
        self.upsert_colliders(scene.collider_handles, scene.colliders)
        if len(getattr(scene, "joints", ())):
            self.upsert_joints(scene.joint_handles, scene.joints)

    # ---- joint constraints ----
    def upsert_joints(self, handles, descs):
        descs = np.ascontiguousarray(descs)
        handles = np.ascontiguousarray(handles)
        self._check(self.L.npgpu_upsert_joints(self.w, len(descs), _ptr(handles, abi.Handle),
                                               _ptr(descs, abi.JointDesc)), "upsert_joints")
        for h in handles:
            self._joints[int(h["index"])] = int(h["generation"])

    def remove_joints(self, handles):
        handles = np.ascontiguousarray(handles)
        self._check(self.L.npgpu_remove_joints(self.w, len(handles), _ptr(handles, abi.Handle)), "remove_joints")
        for h in handles:
            self._joints.pop(int(h["index"]), None)

    def joints(self, handles):
        """(impulses (n, 7): linear, angular, the limit's; broken (n,), active (n,)) after the last step."""
        handles = np.ascontiguousarray(handles)
        out = (abi.JointState * max(len(handles), 1))()
        self._check(self.L.npgpu_get_joints(self.w, len(handles), _ptr(handles, abi.Handle), out), "get_joints")
        n = len(handles)
        imp = np.array([list(out[k].impulses) + [out[k].limit_impulse] for k in range(n)], np.float32).reshape(n, 7)
        broken = np.array([out[k].broken for k in range(n)], bool)
        active = np.array([out[k].active for k in range(n)], bool)
        return imp, broken, active

    def remove_bodies(self, handles):
        handles = np.ascontiguousarray(handles)
        self._check(self.L.npgpu_remove_bodies(self.w, len(handles), _ptr(handles, abi.Handle)), "remove_bodies")

    def remove_colliders(self, handles):
        handles = np.ascontiguousarray(handles)
        self._check(self.L.npgpu_remove_colliders(self.w, len(handles), _ptr(handles, abi.Handle)), "remove_colliders")

    def apply_forces(self, handles, forces, wake=True):
        handles = np.ascontiguousarray(handles)
        f = np.ascontiguousarray(forces, np.float32)
        self._check(self.L.npgpu_apply_forces(self.w, len(handles), _ptr(handles, abi.Handle), _ptr(f, C.c_float),
                                              int(wake)), "apply_forces")

    def step(self, n=1, joints=None, force_generators=0, sync=True):
        """`joints`: the caller's joint-set size (default: the joints uploaded)."""
        if joints is None:
            joints = len(self._joints)
        self._check(self.L.npgpu_step(self.w, n, joints, force_generators), "step")
        if sync:
            self.synchronize()

    def synchronize(self):
        self._check(self.L.npgpu_synchronize(self.w), "synchronize")

    def bodies(self, first=0, n=None):
        n = self.num_bodies - first if n is None else n
        pos = np.zeros((n, 7), np.float32)
        vel = np.zeros((n, 6), np.float32)
        energy = np.zeros(n, np.float32)
        active = np.zeros(n, np.uint8)
        self._check(self.L.npgpu_download_bodies(self.w, first, n, _ptr(pos, C.c_float), _ptr(vel, C.c_float),
                                                 _ptr(energy, C.c_float), _ptr(active, C.c_uint8)), "download_bodies")
        return {"position": pos, "velocity": vel, "energy": energy, "active": active}

    def download_into(self, pos, vel, first=0):
        """Copies positions and velocities into caller-owned host arrays."""
        n = pos.shape[0]
        self._check(self.L.npgpu_download_bodies(self.w, first, n, _ptr(pos, C.c_float), _ptr(vel, C.c_float),
                                                 None, None), "download_bodies")

    def mass_properties(self, first=0, n=None):
        n = self.num_bodies - first if n is None else n
        inertia = np.zeros((n, 7), np.float32)
        com = np.zeros((n, 3), np.float32)
        self._check(self.L.npgpu_download_mass_properties(self.w, first, n, _ptr(inertia, C.c_float),
                                                          _ptr(com, C.c_float)), "mass_properties")
        return inertia, com

    def pairs(self):
        cnt = C.c_uint32(0)
        self._check(self.L.npgpu_get_pairs(self.w, None, 0, C.byref(cnt)), "get_pairs")
        out = np.zeros((max(cnt.value, 1), 2), np.uint32)
        self._check(self.L.npgpu_get_pairs(self.w, _ptr(out, C.c_uint32), cnt.value, C.byref(cnt)), "get_pairs")
        return out[:cnt.value]

    def aabbs(self, first=0, n=None):
        n = self.num_colliders - first if n is None else n
        out = np.zeros((n, 6), np.float32)
        self._check(self.L.npgpu_get_aabbs(self.w, first, n, _ptr(out, C.c_float)), "get_aabbs")
        return out

    def contacts(self):
        cnt = C.c_uint32(0)
        self._check(self.L.npgpu_get_contacts(self.w, None, 0, C.byref(cnt)), "get_contacts")
        n = cnt.value
        arr = (abi.Contact * max(n, 1))()
        self._check(self.L.npgpu_get_contacts(self.w, arr, n, C.byref(cnt)), "get_contacts")
        return abi.contacts_to_numpy(arr, n)

    # ---- geometric queries and contact events ----
    def rays(self, rays6, max_toi, world=abi.ALL_WORLDS):
        """GeometricalWorld::interferences_with_ray for a batch: an array of
        (ray, collider, toi, nx, ny, nz) rows sorted by (ray, collider)."""
        rays6 = np.ascontiguousarray(rays6, np.float32).reshape(-1, 6)
        max_toi = np.ascontiguousarray(max_toi, np.float32).reshape(-1)
        cnt = C.c_uint32(0)
        self._check(self.L.npgpu_interferences_with_rays(self.w, len(rays6), _ptr(rays6, C.c_float),
                                                         _ptr(max_toi, C.c_float), world, None, 0, C.byref(cnt)),
                    "interferences_with_rays")
        n = cnt.value
        arr = (abi.RayHit * max(n, 1))()
        self._check(self.L.npgpu_interferences_with_rays(self.w, len(rays6), _ptr(rays6, C.c_float),
                                                         _ptr(max_toi, C.c_float), world, arr, n, C.byref(cnt)),
                    "interferences_with_rays")
        out = np.zeros((n, 6), np.float64)
        for k in range(n):
            h = arr[k]
            out[k] = (h.ray, h.collider, h.toi, h.normal[0], h.normal[1], h.normal[2])
        return out

    def _pair_query(self, fn, q, per, world):
        q = np.ascontiguousarray(q, np.float32).reshape(-1, per)
        cnt = C.c_uint32(0)
        self._check(fn(self.w, len(q), _ptr(q, C.c_float), world, None, 0, C.byref(cnt)), "interferences")
        out = np.zeros((max(cnt.value, 1), 2), np.uint32)
        self._check(fn(self.w, len(q), _ptr(q, C.c_float), world, _ptr(out, C.c_uint32), cnt.value, C.byref(cnt)),
                    "interferences")
        return out[:cnt.value]

    def points(self, points3, world=abi.ALL_WORLDS):
        """interferences_with_point: (point, collider) rows."""
        return self._pair_query(self.L.npgpu_interferences_with_points, points3, 3, world)

    def aabb_query(self, aabbs6, world=abi.ALL_WORLDS):
        """interferences_with_aabb: (box, collider) rows."""
        return self._pair_query(self.L.npgpu_interferences_with_aabbs, aabbs6, 6, world)

    def enable_contact_events(self, capacity=1 << 20):
        self._check(self.L.npgpu_enable_contact_events(self.w, capacity), "enable_contact_events")

    def contact_events(self):
        """The last step's (collider1, collider2, stopped) rows, sorted."""
        cnt = C.c_uint32(0)
        self._check(self.L.npgpu_contact_events(self.w, None, 0, C.byref(cnt)), "contact_events")
        n = cnt.value
        arr = (abi.ContactEvent * max(n, 1))()
        self._check(self.L.npgpu_contact_events(self.w, arr, n, C.byref(cnt)), "contact_events")
        out = np.zeros((n, 3), np.uint32)
        for k in range(n):
            out[k] = (arr[k].collider1, arr[k].collider2, arr[k].stopped)
        return out

    def proximity_events(self):
        """The last step's (collider1, collider2, previous, new) proximity
        events of pairs with a sensor, by pair and, within a pair, in pass
        order."""
        cnt = C.c_uint32(0)
        self._check(self.L.npgpu_proximity_events(self.w, None, 0, C.byref(cnt)), "proximity_events")
        n = cnt.value
        arr = (abi.ProximityEvent * max(n, 1))()
        self._check(self.L.npgpu_proximity_events(self.w, arr, n, C.byref(cnt)), "proximity_events")
        out = np.zeros((n, 4), np.uint32)
        for k in range(n):
            out[k] = (arr[k].collider1, arr[k].collider2, arr[k].prev_status, arr[k].new_status)
        return out

    def autotune(self, steps_per_candidate=5):
        """Times the solver's launch shapes on real steps (all give the same
        bits) and keeps the fastest: (schedule, world_threads, ms per step)."""
        s, t, ms = C.c_uint32(0), C.c_uint32(0), C.c_float(0.0)
        self._check(self.L.npgpu_autotune(self.w, steps_per_candidate, C.byref(s), C.byref(t), C.byref(ms)),
                    "autotune")
        self.params.solver_schedule = s.value
        self.params.world_threads = t.value
        return s.value, t.value, ms.value

    # ---- learned warm start ----
    def mlp_set(self, params):
        params = np.ascontiguousarray(params, np.float32)
        self._check(self.L.npgpu_mlp_set(self.w, _ptr(params, C.c_float), params.size), "mlp_set")

    def mlp_get(self):
        out = np.zeros(abi.MLP_PARAMS, np.float32)
        self._check(self.L.npgpu_mlp_get(self.w, _ptr(out, C.c_float), out.size), "mlp_get")
        return out

    def mlp_record(self, capacity):
        self._check(self.L.npgpu_mlp_record(self.w, capacity), "mlp_record")

    def mlp_samples(self, download=True):
        n = C.c_uint32(0)
        self._check(self.L.npgpu_mlp_samples(self.w, None, 0, C.byref(n)), "mlp_samples")
        if not download:
            return n.value
        out = np.zeros((n.value, abi.MLP_SAMPLE_FLOATS), np.float32)
        if n.value:
            self._check(self.L.npgpu_mlp_samples(self.w, _ptr(out, C.c_float), n.value, C.byref(n)), "mlp_samples")
        return out

    def mlp_load_samples(self, samples):
        samples = np.ascontiguousarray(samples, np.float32).reshape(-1, abi.MLP_SAMPLE_FLOATS)
        self._check(self.L.npgpu_mlp_load_samples(self.w, _ptr(samples, C.c_float), samples.shape[0]),
                    "mlp_load_samples")

    def mlp_train(self, steps, batch=4096, lr=1e-3, seed=1, init=False):
        loss = C.c_float(0.0)
        self._check(self.L.npgpu_mlp_train(self.w, steps, batch, lr, seed, abi.MLP_INIT if init else 0,
                                           C.byref(loss)), "mlp_train")
        return loss.value

    def mlp_grad(self, samples):
        samples = np.ascontiguousarray(samples, np.float32)
        grad = np.zeros(abi.MLP_TRAINABLE, np.float32)
        loss = C.c_float(0.0)
        self._check(self.L.npgpu_mlp_grad(self.w, _ptr(samples, C.c_float), samples.shape[0], _ptr(grad, C.c_float),
                                          C.byref(loss)), "mlp_grad")
        return grad, loss.value

    def counters(self):
        c = abi.Counters()
        self._check(self.L.npgpu_get_counters(self.w, C.byref(c)), "get_counters")
        return c.as_dict()
