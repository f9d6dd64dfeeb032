"""Reading and writing SHRenderer checkpoints.

The reference writes them with ``torch.save`` (gs/sh_renderer.py:663-679): a
dict of the five parameter tensors (``mean``, ``qvec``,
``svec_before_activation``, ``sh_coeffs``, ``alpha_before_activation``), the
Gaussian count ``N`` and the training configuration ``cfg`` -- a Hydra /
OmegaConf object in the reference's training runs.  Unpickling that object
needs omegaconf, which a serving host need not have, and a pickle can name
any importable callable, which unpickling would run.  So ``load_state``
resolves only the names a tensor checkpoint needs (torch's tensor and storage
rebuild functions, storage classes, ``torch.Size``, dtypes, builtin
containers) and maps every other class -- omegaconf's included -- to an inert
stand-in that keeps its pickled state (the configuration is metadata here;
the tensors are what is served).  Nothing a checkpoint names beyond that
list is imported or called.
"""
from __future__ import annotations

import pickle
from pathlib import Path

import torch

PARAM_KEYS = ("mean", "qvec", "svec_before_activation", "sh_coeffs", "alpha_before_activation")


class Opaque:
    """Stand-in for an object whose class is not importable here; keeps the
    pickled state for inspection."""

    def __init__(self, *args, **kwargs):
        self.__dict__["_args"] = args

    def __setstate__(self, state):
        self.__dict__["_state"] = state

    def __reduce__(self):  # re-saving keeps the stand-in, not the original class
        return (type(self), self.__dict__.get("_args", ()), self.__dict__.get("_state"))


_BUILTINS = {"dict", "list", "tuple", "set", "frozenset", "bytearray", "bytes", "str", "int", "float", "bool",
             "complex", "slice", "range"}


def _allowed(module: str, name: str) -> bool:
    """Names a torch.save checkpoint of tensors needs to be rebuilt."""
    if module == "torch._utils":
        return name.startswith("_rebuild_")
    if module == "torch":
        return name.endswith("Storage") or name == "Size" or isinstance(getattr(torch, name, None), torch.dtype)
    if module == "torch.storage":
        return name in ("TypedStorage", "UntypedStorage")
    if module == "collections":
        return name == "OrderedDict"
    if module == "builtins":
        return name in _BUILTINS
    if module == "_codecs":
        return name == "encode"  # bytes objects pickled with protocol 2
    return False


class _Unpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if _allowed(module, name):
            return super().find_class(module, name)
        return type(name, (Opaque,), {"__module__": "gsx_missing." + module})


class _PickleModule:
    """The subset of the pickle module torch.load uses, with the tolerant
    unpickler."""

    Unpickler = _Unpickler
    __name__ = "gsx_checkpoint_pickle"

    @staticmethod
    def load(f, **kwargs):
        return _Unpickler(f, **kwargs).load()


def load_state(path, device="cpu") -> dict:
    """The checkpoint dict with tensors on `device` (float32, contiguous)."""
    sd = torch.load(Path(path), map_location=device, weights_only=False, pickle_module=_PickleModule)
    missing = [k for k in PARAM_KEYS if k not in sd]
    if missing:
        raise KeyError(f"{path}: not an SHRenderer checkpoint (missing {missing})")
    for k in PARAM_KEYS:
        sd[k] = sd[k].to(device, torch.float32).contiguous()
    n = int(sd.get("N", sd["mean"].shape[0]))
    if n != sd["mean"].shape[0] or any(sd[k].shape[0] != n for k in PARAM_KEYS):
        raise ValueError(f"{path}: inconsistent Gaussian counts")
    sd["N"] = n
    return sd


def save_state(path, mean, qvec, log_scale, sh, alpha_logit, cfg=None) -> None:
    """Write the reference's checkpoint layout."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    torch.save({"mean": mean.detach(), "qvec": qvec.detach(), "svec_before_activation": log_scale.detach(),
                "sh_coeffs": sh.detach(), "alpha_before_activation": alpha_logit.detach(),
                "N": int(mean.shape[0]), "cfg": cfg}, path)
