"""SHRenderer checkpoints (the reference's torch.save layout,
gs/sh_renderer.py:663-708): round trip, a pickled configuration whose class
cannot be imported here (as a Hydra/OmegaConf config is without omegaconf),
and malformed files."""
import pickle
import sys
import types

import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import checkpoint as ck  # noqa: E402
from gaussian_splatting_3d_gb300.sh_renderer import SHRenderer  # noqa: E402


def params(n=7, C=2, seed=0):
    g = torch.Generator().manual_seed(seed)
    return [torch.randn(n, 3, generator=g), torch.randn(n, 4, generator=g), torch.randn(n, 3, generator=g),
            torch.randn(n, 3, C * C, generator=g), torch.randn(n, generator=g)]


def test_round_trip(tmp_path):
    p = params()
    ck.save_state(tmp_path / "a" / "ckpt.pt", *p, cfg={"sh_order": 2})
    sd = ck.load_state(tmp_path / "a" / "ckpt.pt")
    for k, t in zip(ck.PARAM_KEYS, p):
        assert torch.equal(sd[k], t)
    assert sd["N"] == 7 and sd["cfg"] == {"sh_order": 2}


def test_config_of_an_unimportable_class(tmp_path):
    mod = types.ModuleType("fake_hydra_cfg")

    class DictConfig:
        def __init__(self, d):
            self.content = d

    DictConfig.__module__ = "fake_hydra_cfg"
    DictConfig.__qualname__ = "DictConfig"
    mod.DictConfig = DictConfig
    sys.modules["fake_hydra_cfg"] = mod
    try:
        p = params()
        torch.save({"mean": p[0], "qvec": p[1], "svec_before_activation": p[2], "sh_coeffs": p[3],
                    "alpha_before_activation": p[4], "N": 7, "cfg": DictConfig({"tile_size": 16})},
                   tmp_path / "ref.pt", pickle_module=pickle)
    finally:
        del sys.modules["fake_hydra_cfg"]
    sd = ck.load_state(tmp_path / "ref.pt")
    assert isinstance(sd["cfg"], ck.Opaque)
    assert sd["cfg"]._state == {"content": {"tile_size": 16}}
    assert torch.equal(sd["sh_coeffs"], p[3])
    r = SHRenderer.load(tmp_path / "ref.pt", device="cpu")
    assert r.N == 7 and r.max_C == 2 and torch.equal(r.mean.data, p[0])


def test_malformed(tmp_path):
    torch.save({"mean": torch.zeros(3, 3)}, tmp_path / "bad.pt")
    with pytest.raises(KeyError):
        ck.load_state(tmp_path / "bad.pt")
    p = params()
    torch.save({"mean": p[0], "qvec": p[1][:5], "svec_before_activation": p[2], "sh_coeffs": p[3],
                "alpha_before_activation": p[4], "N": 7, "cfg": None}, tmp_path / "bad2.pt")
    with pytest.raises(ValueError):
        ck.load_state(tmp_path / "bad2.pt")


def test_shrenderer_save_load(tmp_path):
    r = SHRenderer(None, device="cpu", sh_order=2)
    p = params()
    r.N = 7
    for k, t in zip(ck.PARAM_KEYS, p):
        setattr(r, k, torch.nn.Parameter(t))
    r.save(tmp_path / "s.pt")
    q = SHRenderer.load(tmp_path / "s.pt", device="cpu")
    for k in ck.PARAM_KEYS:
        assert torch.equal(getattr(q, k).data, getattr(r, k).data)


class _RunsCode:
    """Pickles as a call of an importable function (here ``os.getpid`` on
    load): a checkpoint must not be able to make the loader call it."""

    def __reduce__(self):
        import os

        return (os.getpid, ())


def test_checkpoint_cannot_call_importable_functions(tmp_path):
    p = params()
    torch.save({"mean": p[0], "qvec": p[1], "svec_before_activation": p[2], "sh_coeffs": p[3],
                "alpha_before_activation": p[4], "N": 7, "cfg": _RunsCode()}, tmp_path / "evil.pt",
               pickle_module=pickle)
    sd = ck.load_state(tmp_path / "evil.pt")
    # the named function was replaced by an inert stand-in, not called
    assert isinstance(sd["cfg"], ck.Opaque)
    assert type(sd["cfg"]).__module__.startswith("gsx_missing.")
    assert torch.equal(sd["mean"], p[0])
