"""Drop-in for the reference's galaxy_formation/engine.py: the same `Engine` API, backed by
libgfgpu.so (GB300 CUDA kernels) instead of cpp/nbody.cpp.

`Engine.gravity` / `gravity_direct` / `project` / `tonemap` keep the reference's
signatures and NumPy in/out semantics (galaxy_formation/engine.py:45-72). `gravity` and
`gravity_direct` also accept torch CUDA tensors, in which case the device-resident entry
points are used on torch's current stream and nothing crosses PCIe/C2C.
"""

import numpy as np

from . import _lib


def _is_cuda_tensor(x):
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _stream_ptr():
    import torch

    # torch's default stream is the legacy default stream (handle 0); the library reads NULL
    # as its own stream, so the legacy stream goes as cudaStreamLegacy ((cudaStream_t)1)
    return torch.cuda.current_stream().cuda_stream or 1


class Engine:
    """Typed interface to the GPU library (galaxy_formation/engine.py:39-72)."""

    def __init__(self):
        self.lib = _lib.load()
        if self.lib.nbody_num_threads() <= 0:
            raise _lib.GpuError(64, "no usable CUDA device")

    def gravity(self, pos, mass, acc, theta, eps, active=None, rebuild=True):
        """acc[i] = the Barnes-Hut acceleration (G = 1, Plummer eps, opening angle theta) of
        every particle with active[i] (all when active is None); other rows are not touched.
        rebuild=False keeps the tree of the last call and refreshes its moments."""
        n = len(mass)
        if _is_cuda_tensor(pos):
            act = 0 if active is None else active.data_ptr()
            st = self.lib.gf_accel_active_dev(n, pos.data_ptr(), mass.data_ptr(), acc.data_ptr(),
                                              float(theta), float(eps), act, int(rebuild),
                                              _stream_ptr())
            _lib.check(st)
            return
        act = np.ones(n, np.uint8) if active is None else np.ascontiguousarray(active, dtype=np.uint8)
        self.lib.nbody_accel_active(n, pos, mass, acc, theta, eps, act, int(rebuild))
        _lib.check()

    def gravity_direct(self, pos, mass, eps):
        """The float64 pairwise sum over all particles, O(N^2): the exact reference."""
        if _is_cuda_tensor(pos):
            import torch

            acc = torch.zeros_like(pos)
            st = self.lib.gf_accel_direct_dev(len(mass), pos.data_ptr(), mass.data_ptr(),
                                              acc.data_ptr(), float(eps), _stream_ptr())
            _lib.check(st)
            return acc
        acc = np.zeros_like(pos)
        self.lib.nbody_accel_direct(len(mass), pos, mass, acc, eps)
        _lib.check()
        return acc

    def gravity_direct_targets(self, pos, mass, targets, eps):
        """Exact accelerations of the particles `targets` only, shape (len(targets), 3)."""
        t = np.ascontiguousarray(targets, dtype=np.int64)
        acc = np.zeros((len(t), 3))
        _lib.check(self.lib.gf_accel_direct_targets(len(mass), pos, mass, len(t), t, acc, eps))
        return acc

    def project(self, pos, group, n_groups, rot, scale, size):
        """Splats the particles into one float32 image per colour group, (n_groups, size, size):
        orthographic view through rot, `scale` pixels per length unit, bilinear weights."""
        img = np.empty((n_groups, size, size), np.float32)
        self.lib.nbody_render(len(group), np.ascontiguousarray(pos), group, n_groups,
                              np.ascontiguousarray(rot), np.zeros(3), scale, size, size, img)
        _lib.check()
        return img

    def tonemap(self, img, glow, colors, inv_ref, K, exposure):
        """Combines the group images and their quarter-size glow maps into (H, W, 3) uint8:
        logarithmic brightness plus glow, tinted by the group colours, soft-saturated."""
        ng, H, W = img.shape
        out = np.empty((H, W, 3), np.uint8)
        self.lib.nbody_tonemap(W, H, ng, img, np.ascontiguousarray(glow), glow.shape[2], glow.shape[1],
                               np.ascontiguousarray(colors, dtype=np.float32).ravel(),
                               inv_ref, K, exposure, out)
        _lib.check()
        return out

    def tree(self):
        """The current gravity octree in the reference's depth-first layout (test hook)."""
        import ctypes

        nn, ng = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.gf_tree_size(ctypes.byref(nn), ctypes.byref(ng)))
        n = self._n_last
        ints = np.zeros((nn.value, 4), np.int32)
        floats = np.zeros((nn.value, 9), np.float32)
        order = np.zeros(n, np.int32)
        groups = np.zeros(ng.value, np.int32)
        _lib.check(self.lib.gf_tree_export(ints, floats, order, groups))
        return {"start": ints[:, 0], "count": ints[:, 1], "next": ints[:, 2], "leaf": ints[:, 3],
                "cx": floats[:, 0], "cy": floats[:, 1], "cz": floats[:, 2], "m": floats[:, 3],
                "open_r": floats[:, 4], "gx": floats[:, 5], "gy": floats[:, 6], "gz": floats[:, 7],
                "half": floats[:, 8], "order": order, "groups": groups}

    def build_tree(self, pos, mass, theta):
        """Builds the gravity tree without evaluating any acceleration (test hook)."""
        self._n_last = len(mass)
        acc = np.zeros_like(pos)
        self.gravity(pos, mass, acc, theta, 0.1, np.zeros(len(mass), np.uint8), True)
        return self.tree()
