"""Minimal stand-in for the ``autoray`` package, used only to import the
unmodified reference torchquad in a container where ``autoray`` is not
installed, so that ``tests/golden/make_golden.py`` can record the reference's
outputs as golden fixtures.

autoray itself does no arithmetic: it forwards numpy-style calls to the
backend library.  This shim does the same for the two backends the fixtures
need (torch and numpy), translating numpy argument names (``axis``) and
function names (``concatenate``) to their torch spellings.  Test
infrastructure only; nothing in the product imports it.
"""
import builtins
import numpy as _np

_REGISTRY = {}

# numpy name -> torch name
_TORCH_NAMES = {
    "array": "tensor",
    "asarray": "as_tensor",
    "concatenate": "cat",
    "equal": "eq",
    "multiply": "mul",
    "power": "pow",
    "logical_not": "logical_not",
    "array_equal": "equal",
}


def infer_backend(x):
    mod = type(x).__module__.split(".")[0]
    if mod == "numpy":
        return "numpy"
    return mod


def _backend_of(args, kwargs):
    like = kwargs.pop("like", None)
    if like is not None:
        return like if isinstance(like, str) else infer_backend(like)
    for a in list(args) + list(kwargs.values()):
        b = infer_backend(a)
        if b in ("torch", "numpy"):
            return b
        if isinstance(a, (list, tuple)) and len(a) > 0:
            b = infer_backend(a[0])
            if b in ("torch", "numpy"):
                return b
    return "numpy"


def _torch_call(name, args, kwargs):
    import torch

    if "axis" in kwargs:
        kwargs["dim"] = kwargs.pop("axis")
    if name == "array":
        x = args[0]
        dtype = kwargs.get("dtype", None)
        if isinstance(dtype, str):
            dtype = getattr(torch, dtype)
        if isinstance(x, torch.Tensor):
            return x.to(dtype) if dtype is not None else x
        if isinstance(x, (list, tuple)) and len(x) > 0 and isinstance(x[0], torch.Tensor):
            t = torch.stack(list(x))
            return t.to(dtype) if dtype is not None else t
        return torch.tensor(x, dtype=dtype)
    if name in ("zeros", "ones", "linspace", "arange") and isinstance(kwargs.get("dtype"), str):
        kwargs["dtype"] = getattr(torch, kwargs["dtype"])
    if name in ("sum", "prod", "max", "min") and kwargs.get("dim", 0) is None:
        kwargs.pop("dim")
    if name in ("max", "min") and "dim" in kwargs:
        return getattr(torch, "amax" if name == "max" else "amin")(*args, **kwargs)
    if name == "meshgrid":
        return torch.meshgrid(*args, **kwargs)
    if name == "squeeze" and "dim" not in kwargs:
        return torch.squeeze(args[0])
    tname = _TORCH_NAMES.get(name, name)
    return getattr(torch, tname)(*args, **kwargs)


def do(name, *args, **kwargs):
    backend = _backend_of(args, kwargs)
    fn = _REGISTRY.get((backend, name))
    if fn is not None:
        return fn(*args, **kwargs)
    if backend == "torch":
        return _torch_call(name, args, kwargs)
    if backend == "numpy":
        kwargs.pop("dim", None)
        return getattr(_np, name)(*args, **kwargs)
    return getattr(builtins, name)(*args, **kwargs)


class _Namespace:
    def __init__(self, prefix=""):
        self._prefix = prefix

    def __getattr__(self, name):
        if name == "random":
            return _Namespace("random.")
        if name == "ndarray":
            return _np.ndarray
        full = self._prefix + name

        def call(*args, **kwargs):
            return do(full, *args, **kwargs)

        return call


numpy = _Namespace()


def register_function(backend, name, fn=None):
    if fn is None:

        def deco(f):
            _REGISTRY[(backend, name)] = f
            return f

        return deco
    _REGISTRY[(backend, name)] = fn
    return fn


def to_backend_dtype(dtype_name, like):
    backend = like if isinstance(like, str) else infer_backend(like)
    if backend == "torch":
        import torch

        return getattr(torch, dtype_name)
    return _np.dtype(dtype_name)


def get_dtype_name(x):
    d = x.dtype if hasattr(x, "dtype") else x
    return str(d).replace("torch.", "")


def astype(x, dtype):
    if infer_backend(x) == "torch":
        import torch

        if isinstance(dtype, str):
            dtype = getattr(torch, dtype)
        return x.to(dtype)
    return x.astype(dtype)


def to_numpy(x):
    if infer_backend(x) == "torch":
        return x.detach().cpu().numpy()
    return _np.asarray(x)
