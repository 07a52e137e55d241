"""Learned coarse-grid correction (host side).

A small 2D convolutional encoder-decoder replaces the multigrid coarse-grid
correction below one level of the shifted-Laplacian cycle.  Its forward and
backward passes, loss and Adam steps are the library's own CUDA kernels
(``csrc/hz_learn.cu``, BF16 tensor-core convolutions with FP32 accumulation);
this module only drives them through the C ABI:

* ``CoarseNet``: create / weights / forward / gradient / train;
* ``collect_pairs``: (residual, error) pairs from the FP64 solver on one level;
* ``attach``: use a network inside FGMRES, with the plain cycle as the fallback
  when a restart cycle stagnates.

Array layout: ``x`` (batch, ny, nx, 4) float32 = (Re r/s, Im r/s, w^2 m hx hy,
gamma / w) with s the RMS of r; ``t`` / ``y`` (batch, ny, nx, 2) float32 =
e / (hx hy s).  nx runs along the mesh's first axis (the fastest index); node
counts per axis must be 8k+1.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .api import (ShiftedLaplacianMultigridSolver, _device_inputs_ready, _ensure_handle, _is_device_array, _nodes,
                  current_device)


def num_params() -> int:
    return int(L.load().hz_net_num_params())


def num_params_3d() -> int:
    return int(L.load().hz_net3d_num_params())


def layer_shapes_3d() -> list[tuple[int, int]]:
    lib = L.load()
    out = []
    for k in range(6):
        a, b = C.c_int32(), C.c_int32()
        L.check(lib.hz_net3d_layer_shape(k, C.byref(a), C.byref(b)))
        out.append((a.value, b.value))
    return out


def layer_shapes() -> list[tuple[int, int]]:
    lib = L.load()
    out = []
    for k in range(8):
        a, b = C.c_int32(), C.c_int32()
        L.check(lib.hz_net_layer_shape(k, C.byref(a), C.byref(b)))
        out.append((a.value, b.value))
    return out


def _ptr(a):
    """(pointer, mem) of a float32 array on the host (numpy) or a CUDA tensor."""
    if _is_device_array(a):
        if not a.is_contiguous():
            raise ValueError("device arrays must be contiguous")
        _device_inputs_ready()
        return a.data_ptr(), L.HZ_MEM_DEVICE
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        raise ValueError("host arrays must be C-contiguous float32")
    return a.ctypes.data, L.HZ_MEM_HOST


class CoarseNet:
    """The network on one CUDA device (seeded He-normal initial weights)."""

    def __init__(self, seed: int = 0, device: int | None = None):
        """device: CUDA device index (None: the process's current device, as for solver handles)."""
        device = current_device() if device is None else int(device)
        self._h = C.c_void_p()
        L.check(L.load().hz_net_create(int(seed), device, C.byref(self._h)))
        self.device = device

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            L.load().hz_net_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    dim = 2

    def _nparams(self) -> int:
        return num_params()

    def get_weights(self) -> np.ndarray:
        w = np.empty(self._nparams(), dtype=np.float32)
        L.check(L.load().hz_net_get_weights(self._h, w.ctypes.data))
        return w

    def set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.size != self._nparams():
            raise ValueError(f"expected {self._nparams()} weights, got {w.size}")
        L.check(L.load().hz_net_set_weights(self._h, w.ctypes.data))

    def forward(self, x):
        """y = net(x); x (batch, ny, nx, 4) numpy float32 or CUDA tensor."""
        B, ny, nx, c = x.shape
        if c != 4:
            raise ValueError("x must have 4 channels")
        if _is_device_array(x):
            import torch
            y = torch.empty((B, ny, nx, 2), dtype=torch.float32, device=x.device)
        else:
            y = np.empty((B, ny, nx, 2), dtype=np.float32)
        px, mem = _ptr(x)
        py, _ = _ptr(y)
        L.check(L.load().hz_net_forward(self._h, px, py, nx, ny, B, mem))
        return y

    def gradient(self, x, t):
        """(loss, weight gradient as a flat float32 array) for one batch."""
        B, ny, nx, _ = x.shape
        px, mem = _ptr(x)
        pt, mem2 = _ptr(t)
        if mem != mem2:
            raise ValueError("x and t must both be on the host or both on the device")
        g = np.empty(num_params(), dtype=np.float32)
        loss = C.c_double()
        L.check(L.load().hz_net_gradient(self._h, px, pt, nx, ny, B, mem, C.byref(loss), g.ctypes.data))
        return loss.value, g

    def save(self, path) -> None:
        """Weights and Adam state to a versioned binary file (training resumes from it)."""
        L.check(L.load().hz_net_save(self._h, str(path).encode()))

    def load(self, path) -> None:
        """Weights and Adam state from a file written by save (format, version and shapes checked)."""
        L.check(L.load().hz_net_load(self._h, str(path).encode()))

    def set_conv_path(self, path: str) -> None:
        """Convolution kernels: "mma" (warp-level mma.sync), "tcgen05" (5th-generation
        tensor cores with the accumulator in tensor memory and the operands staged
        by the TMA unit, every layer they support) or "auto" (the default: per layer
        the faster of the two)."""
        code = {"mma": L.HZ_NET_CONV_WARP_MMA, "tcgen05": L.HZ_NET_CONV_TCGEN05, "auto": L.HZ_NET_CONV_AUTO}[path]
        L.check(L.load().hz_net_set_conv_path(self._h, code))

    def set_profile(self, on: bool) -> None:
        """Time every kernel launch of the network's own stream with CUDA events."""
        L.check(L.load().hz_net_set_profile(self._h, int(bool(on))))

    def kernel_times(self) -> list[dict]:
        """Launch table of the network's stream: name, launches, timed launches,
        milliseconds, algorithmic bytes and flops per kernel."""
        lib = L.load()
        n = lib.hz_net_kernel_times(self._h, -1, None, 0, None, None, None, None, None)
        rows = []
        for i in range(n):
            name = C.create_string_buffer(64)
            la, lt = C.c_int64(), C.c_int64()
            ms, by, fl = C.c_double(), C.c_double(), C.c_double()
            lib.hz_net_kernel_times(self._h, i, name, 64, C.byref(la), C.byref(lt), C.byref(ms), C.byref(by),
                                    C.byref(fl))
            rows.append(dict(name=name.value.decode(), launches=la.value, timed=lt.value, ms=ms.value,
                             bytes=by.value, flops=fl.value))
        return rows

    def reset_kernel_times(self) -> None:
        L.check(L.load().hz_net_reset_kernel_times(self._h))

    def train(self, x, t, epochs: int = 10, batch: int = 32, lr: float = 2e-3, seed: int = 0) -> np.ndarray:
        """Adam over the pairs (CUDA tensors) for epochs passes; returns the mean loss per epoch."""
        if not (_is_device_array(x) and _is_device_array(t)):
            raise ValueError("training pairs must be CUDA tensors")
        P, ny, nx, _ = x.shape
        hist = np.zeros(int(epochs))
        _device_inputs_ready()
        L.check(L.load().hz_net_train(self._h, x.data_ptr(), t.data_ptr(), nx, ny, P, int(batch), int(epochs),
                                      float(lr), int(seed), hist.ctypes.data_as(C.POINTER(C.c_double))))
        return hist


class CoarseNet3D(CoarseNet):
    """The 3D network (three grid levels, 8-16-32 channels, 3x3x3 convolutions) on
    one CUDA device; arrays are (batch, nz, ny, nx, channels) with node counts 4k+1."""

    dim = 3

    def __init__(self, seed: int = 0, device: int | None = None):
        device = current_device() if device is None else int(device)
        self._h = C.c_void_p()
        L.check(L.load().hz_net3d_create(int(seed), device, C.byref(self._h)))
        self.device = device

    def _nparams(self) -> int:
        return num_params_3d()

    def forward(self, x):
        """y = net(x); x (batch, nz, ny, nx, 4) numpy float32 or CUDA tensor."""
        B, nz, ny, nx, c = x.shape
        if c != 4:
            raise ValueError("x must have 4 channels")
        if _is_device_array(x):
            import torch
            y = torch.empty((B, nz, ny, nx, 2), dtype=torch.float32, device=x.device)
        else:
            y = np.empty((B, nz, ny, nx, 2), dtype=np.float32)
        px, mem = _ptr(x)
        py, _ = _ptr(y)
        L.check(L.load().hz_net3d_forward(self._h, px, py, nx, ny, nz, B, mem))
        return y

    def gradient(self, x, t):
        """(loss, weight gradient as a flat float32 array) for one batch."""
        B, nz, ny, nx, _ = x.shape
        px, mem = _ptr(x)
        pt, mem2 = _ptr(t)
        if mem != mem2:
            raise ValueError("x and t must both be on the host or both on the device")
        g = np.empty(self._nparams(), dtype=np.float32)
        loss = C.c_double()
        L.check(L.load().hz_net3d_gradient(self._h, px, pt, nx, ny, nz, B, mem, C.byref(loss), g.ctypes.data))
        return loss.value, g

    def train(self, x, t, epochs: int = 10, batch: int = 8, lr: float = 2e-3, seed: int = 0) -> np.ndarray:
        """Adam over the pairs (CUDA tensors) for epochs passes; returns the mean loss per epoch."""
        if not (_is_device_array(x) and _is_device_array(t)):
            raise ValueError("training pairs must be CUDA tensors")
        P, nz, ny, nx, _ = x.shape
        hist = np.zeros(int(epochs))
        _device_inputs_ready()
        L.check(L.load().hz_net3d_train(self._h, x.data_ptr(), t.data_ptr(), nx, ny, nz, P, int(batch), int(epochs),
                                        float(lr), int(seed), hist.ctypes.data_as(C.POINTER(C.c_double))))
        return hist


def file_info(path) -> tuple[int, int]:
    """(parameter count, Adam step) of a saved network file; raises for a file
    that is not loadable (host only, no GPU)."""
    n, st = C.c_int64(), C.c_int64()
    L.check(L.load().hz_net_file_info(str(path).encode(), C.byref(n), C.byref(st)))
    return int(n.value), int(st.value)


def level_grid(solver: ShiftedLaplacianMultigridSolver, level: int) -> tuple[int, ...]:
    """Node counts (nx, ny) or (nx, ny, nz) of a multigrid level."""
    nodes = [int(v) for v in _nodes(solver.helmParam.Mesh)]
    for _ in range(level):
        nodes = [(v - 1) // 2 + 1 for v in nodes]
    return tuple(nodes)


def collect_pairs(solver: ShiftedLaplacianMultigridSolver, B, level: int = 2, sweeps: int = 2,
                  max_pairs: int | None = None):
    """Training pairs from the FP64 solver (see hz_collect_pairs).

    B: (n, nrhs) complex right-hand sides on the host.  Returns a dict with
    ``x``, ``t`` (CUDA tensors, layout above; 3D: (pairs, nz, ny, nx, c)),
    ``plain_err`` (numpy: relative error of the plain coarse correction on each
    pair), ``target_relres`` and ``X`` (the solution of the solve that produced
    them).  2D targets: band LU + (sweeps - 1) refinement steps; 3D targets:
    `sweeps` restarted plain corrections."""
    import torch
    if solver.MG.precision != "fp64":
        raise ValueError("pairs come from the FP64 solver (precision='fp64')")
    Bc = np.asarray(B, dtype=np.complex128)
    if Bc.ndim == 1:
        Bc = Bc.reshape(-1, 1)
    n, nrhs = Bc.shape
    grid = level_grid(solver, level)[::-1]  # (ny, nx) or (nz, ny, nx)
    if max_pairs is None:
        max_pairs = nrhs * solver.MG.maxOuterIter * max(1, solver.inner)
    h = _ensure_handle(solver)
    dev = torch.device("cuda", solver._device)
    x = torch.empty((max_pairs, *grid, 4), dtype=torch.float32, device=dev)
    t = torch.empty((max_pairs, *grid, 2), dtype=torch.float32, device=dev)
    pe = np.zeros(max_pairs)
    rr = C.c_double()
    cnt = C.c_int64()
    Bf = np.asfortranarray(Bc)
    Xf = np.empty((n, nrhs), dtype=np.complex128, order="F")
    code = L.load().hz_collect_pairs(h, Bf.ctypes.data, Xf.ctypes.data, n, nrhs, L.HZ_MEM_HOST, int(level),
                                     int(sweeps), int(max_pairs), x.data_ptr(), t.data_ptr(),
                                     pe.ctypes.data_as(C.POINTER(C.c_double)), C.byref(rr), C.byref(cnt))
    L.check(code, h)
    k = int(cnt.value)
    return dict(x=x[:k], t=t[:k], plain_err=pe[:k], target_relres=rr.value, X=Xf)


def attach(solver: ShiftedLaplacianMultigridSolver, net: CoarseNet | None, level: int = 2,
           stag_ratio: float = 0.95) -> None:
    """Use `net` for the coarse-grid correction of `level` in every later solve
    (FGMRES only); net=None detaches.  A restart cycle that reduces a column's
    residual by less than stag_ratio hands that solve to the plain cycle."""
    solver.learned = None if net is None else (net, int(level), float(stag_ratio))
    if solver._handle is not None:
        _apply(solver)


def _apply(solver: ShiftedLaplacianMultigridSolver) -> None:
    lib = L.load()
    h = solver._handle
    if solver.learned is None:
        L.check(lib.hz_attach_net(h, None, 0, 1.0), h)
    else:
        net, level, stag = solver.learned
        L.check(lib.hz_attach_net(h, net._h, level, stag), h)


def learned_stats(solver: ShiftedLaplacianMultigridSolver) -> tuple[int, int]:
    """(network applications, fallbacks to the plain cycle) of the solver's handle."""
    if solver._handle is None:
        return 0, 0
    calls, fb = C.c_int64(), C.c_int32()
    L.check(L.load().hz_learned_stats(solver._handle, C.byref(calls), C.byref(fb)), solver._handle)
    return int(calls.value), int(fb.value)


def pair_errors(net: CoarseNet, x, t, batch: int = 64) -> np.ndarray:
    """Relative error ||net(x) - t|| / ||t|| per pair (CUDA tensors)."""
    import torch
    out = []
    for i in range(0, x.shape[0], batch):
        y = net.forward(x[i:i + batch].contiguous())
        tt = t[i:i + batch]
        num = torch.linalg.vector_norm((y - tt).reshape(y.shape[0], -1), dim=1)
        den = torch.linalg.vector_norm(tt.reshape(y.shape[0], -1), dim=1)
        out.append((num / den).double().cpu().numpy())
    return np.concatenate(out) if out else np.zeros(0)
