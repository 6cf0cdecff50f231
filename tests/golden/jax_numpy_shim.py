"""A NumPy-backed stand-in for the parts of ``jax`` the l3es hot path touches.

Used only by ``make_golden.py`` to run the reference's own source files in a
container where jax/jaxlib 0.4.29 are not installed. The reference enables x64
(l3es/spectral_solver.py:24), so FP64 NumPy arithmetic is the same precision.
Covered: ``jax.numpy`` (delegating to numpy, with ``x.at[idx].set/add``),
``jax.config``, ``jax.lax.scan``, ``jax.vmap``, ``jax.jit`` (identity),
``jax.ops.segment_sum`` and import
stubs for the unavailable third-party packages (jax_cfd, jax_sph, finufft,
matplotlib), whose functions are never called on the fixture paths.
"""

from __future__ import annotations

import sys
import types

import numpy as np


class JArr(np.ndarray):
    """ndarray with the functional ``.at[idx].set(v)`` / ``.add(v)`` of jax."""

    def block_until_ready(self):
        return self

    @property
    def at(self):
        arr = self

        class _Idx:
            def __getitem__(self, idx):
                class _Op:
                    def set(self, v):
                        out = np.array(arr, copy=True).view(JArr)
                        out[idx] = v
                        return out

                    def add(self, v):
                        out = np.array(arr, copy=True).view(JArr)
                        np.add.at(out, idx, v)
                        return out

                return _Op()

        return _Idx()


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArr):
        return x.view(JArr)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


def _wrapped(fn):
    def f(*a, **k):
        return _wrap(fn(*a, **k))

    return f


class _NPModule(types.ModuleType):
    def __init__(self, name, target):
        super().__init__(name)
        self._target = target

    def __getattr__(self, item):
        obj = getattr(self._target, item)
        if callable(obj) and not isinstance(obj, type):
            return _wrapped(obj)
        return obj


def _scan(f, init, xs):
    carry, ys = init, []
    for x in xs:
        carry, y = f(carry, x)
        ys.append(y)
    return carry, _wrap(np.stack(ys))


def _vmap(f, in_axes=0):
    def g(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = next(a.shape[ax] for a, ax in zip(args, axes) if ax is not None)
        outs = []
        for i in range(n):
            sub = [a if ax is None else np.take(a, i, axis=ax) for a, ax in zip(args, axes)]
            outs.append(f(*sub))
        if isinstance(outs[0], dict):  # a pytree of arrays, as jax.vmap returns it
            return {k: _wrap(np.stack([o[k] for o in outs])) for k in outs[0]}
        if isinstance(outs[0], tuple):
            return tuple(
                None if outs[0][j] is None else _wrap(np.stack([o[j] for o in outs]))
                for j in range(len(outs[0]))
            )
        return _wrap(np.stack(outs))

    return g


def install() -> None:
    """Register the stand-in modules in ``sys.modules``."""
    jax = types.ModuleType("jax")
    jnp = _NPModule("jax.numpy", np)
    jnp.fft = _NPModule("jax.numpy.fft", np.fft)
    jnp.linalg = _NPModule("jax.numpy.linalg", np.linalg)
    jax.numpy = jnp

    class _Cfg:
        def update(self, *a, **k):
            pass

    jax.config = _Cfg()
    lax = types.ModuleType("jax.lax")
    lax.scan = _scan
    jax.lax = lax
    jax.vmap = _vmap
    jax.jit = lambda f, *a, **k: f
    jax.random = types.ModuleType("jax.random")
    jax.ops = types.ModuleType("jax.ops")

    def _segment_sum(data, segment_ids, num_segments):
        data = np.asarray(data)
        out = np.zeros((num_segments,) + data.shape[1:], dtype=data.dtype)
        ids = np.asarray(segment_ids)
        keep = (ids >= 0) & (ids < num_segments)  # jax drops out-of-range ids
        np.add.at(out, ids[keep], data[keep])
        return _wrap(out)

    jax.ops.segment_sum = _segment_sum
    jax.lib = types.SimpleNamespace(
        xla_bridge=types.SimpleNamespace(
            get_backend=lambda: types.SimpleNamespace(platform="cpu")
        )
    )
    jsp = types.ModuleType("jax.scipy")
    jsp.special = types.ModuleType("jax.scipy.special")
    import math

    jsp.special.factorial = lambda n, exact=False: float(math.factorial(int(n)))
    jax.scipy = jsp
    exp = types.ModuleType("jax.experimental")
    exp.serialize_executable = types.ModuleType("jax.experimental.serialize_executable")
    jax.experimental = exp
    for name, mod in {
        "jax": jax,
        "jax.numpy": jnp,
        "jax.numpy.fft": jnp.fft,
        "jax.lax": lax,
        "jax.random": jax.random,
        "jax.ops": jax.ops,
        "jax.experimental": exp,
        "jax.scipy": jsp,
        "jax.scipy.special": jsp.special,
        "jax.experimental.serialize_executable": exp.serialize_executable,
    }.items():
        sys.modules[name] = mod

    def _stub(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    anything = type("Anything", (), {"__getattr__": lambda self, k: self,
                                     "__call__": lambda self, *a, **k: self})()
    for name in [
        "jax_cfd", "jax_cfd.base", "jax_cfd.collocated",
        "jax_sph", "jax_sph.jax_md", "jax_sph.kernel", "jax_sph.partition",
        "jax_sph.utils", "jax_sph.io_state", "jax_sph.eos", "finufft", "seaborn",
        "matplotlib", "matplotlib.pyplot", "matplotlib.cm", "matplotlib.colors",
    ]:
        _stub(name)
    sys.modules["jax_cfd.base"].grids = anything
    sys.modules["jax_cfd.collocated"].initial_conditions = anything
    sys.modules["jax_cfd.collocated"].pressure = anything
    sys.modules["jax_sph.jax_md"].space = anything
    sys.modules["jax_sph.kernel"].QuinticKernel = anything
    sys.modules["jax_sph.eos"].TaitEoS = anything
    sys.modules["jax_sph.partition"].neighbor_list = anything
    sys.modules["jax_sph.utils"].pos_init_cartesian_2d = anything
    sys.modules["jax_sph.utils"].pos_init_cartesian_3d = anything
    sys.modules["jax_sph.io_state"].read_h5 = anything
    sys.modules["jax_sph.io_state"].write_h5 = anything
    for k in ["figure", "subplots", "savefig", "close", "imshow", "colorbar"]:
        setattr(sys.modules["matplotlib.pyplot"], k, anything)
    sys.modules["matplotlib"].use = lambda *a, **k: None
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
