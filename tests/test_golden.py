"""Golden fixtures (tests/golden/oracle_golden.npz, made by make_golden.py):
stored inputs and SHA-256 digests of all eight fields after N Steps.  The CPU
test freezes the oracle; the GPU test holds the CUDA path to the same bits."""
import os

import numpy as np
import pytest

from aeroflux_gb300 import Config, New
from oracle.oracle import OracleEngine
from tests.golden.make_golden import CASES, digest
from tests.helpers import FIELDS, oracle_kwargs

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))


def _inputs(name):
    return GOLD[f"{name}/u"], GOLD[f"{name}/v"], GOLD[f"{name}/w"]


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_reproduces_golden(name):
    kw, kind, _, steps = CASES[name]
    cfg = Config(**kw)
    u, v, w = _inputs(name)
    with OracleEngine(**oracle_kwargs(cfg)) as o:
        o.data(1)[:] = u
        o.data(2)[:] = v
        o.data(3)[:] = w
        if kind != "shear":
            o.apply_velocity_bc()
        o.step(int(GOLD[f"{name}/steps"]))
        got = [digest(o.data(i)) for i in range(8)]
        assert got == list(GOLD[f"{name}/digests"])
        assert o.max_divergence() == float(GOLD[f"{name}/max_divergence"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_reproduces_golden(name):
    kw, kind, _, _ = CASES[name]
    e = New(Config(**kw))
    u, v, w = _inputs(name)
    e.upload("U", u)
    e.upload("V", v)
    e.upload("W", w)
    if kind != "shear":
        e.applyVelocityBC()
    e.Step(int(GOLD[f"{name}/steps"]))
    got = [digest(e.download(n)) for n in FIELDS]
    assert got == list(GOLD[f"{name}/digests"])
    assert e.MaxDivergence() == float(GOLD[f"{name}/max_divergence"])
    ke, ref = e.KineticEnergy(), float(GOLD[f"{name}/kinetic_energy"])
    assert abs(ke - ref) <= 1e-12 * abs(ref)
    e.Close()
