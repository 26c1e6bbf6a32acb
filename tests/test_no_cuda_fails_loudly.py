"""The product path has no CPU fallback: on a host without a CUDA device every
public sampling and pricing call raises, and a missing libtqf.so raises at
load time (CPU)."""

import os
import subprocess
import sys

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")


def _calls():
    from tqf.math import qmc
    from tqf.math.random import RandomType, halton, sobol
    from tqf.models import (GenericItoProcess, GeometricBrownianMotion, HestonModel,
                            MultivariateGeometricBrownianMotion, euler_sampling, milstein_sampling)
    from tqf.models.hjm import GaussianHJM
    from tqf.models.hull_white import HullWhiteModel1F
    from tqf.pricing import basket_european_mc, heston_european_mc
    stateless = dict(seed=[1, 2], random_type=RandomType.STATELESS)
    flat = lambda *args: [0.01]  # noqa: E731
    return {
        "sobol.sample": lambda: sobol.sample(2, 5),
        "halton.sample": lambda: halton.sample(2, 5, seed=1),
        "qmc.lattice_rule_sample": lambda: qmc.lattice_rule_sample(np.array([1, 3], np.int64), 2, 8),
        "euler_sampling.sample": lambda: euler_sampling.sample(
            1, lambda t, x: 0.05 * x, lambda t, x: 0.2 * x[..., None], [1.0], num_time_steps=4, num_samples=4,
            initial_state=[1.0], **stateless),
        "GenericItoProcess.sample_paths": lambda: GenericItoProcess(
            1, lambda t, x: 0.05 * x, lambda t, x: 0.2 * x[..., None]).sample_paths(
            [1.0], num_samples=4, initial_state=[1.0], num_time_steps=4, **stateless),
        "milstein_sampling.sample": lambda: milstein_sampling.sample(
            dim=1, drift_fn=lambda t, x: 0.05 * x, volatility_fn=lambda t, x: 0.2 * x[..., None], times=[1.0],
            num_time_steps=4, num_samples=4, initial_state=[1.0], **stateless),
        "HestonModel.sample_paths": lambda: HestonModel(2.0, 0.04, 0.3, -0.7).sample_paths(
            [1.0], [np.log(100.0), 0.04], 4, num_time_steps=4, **stateless),
        "GeometricBrownianMotion.sample_paths": lambda: GeometricBrownianMotion(0.05, 0.2).sample_paths(
            [1.0], initial_state=1.0, num_samples=4, **stateless),
        "MultivariateGeometricBrownianMotion.sample_paths": lambda: MultivariateGeometricBrownianMotion(
            2, means=[0.05, 0.05], volatilities=[0.2, 0.3], corr_matrix=[[1.0, 0.5], [0.5, 1.0]]).sample_paths(
            [1.0], initial_state=[1.0, 1.0], num_samples=4, **stateless),
        "HullWhiteModel1F.sample_paths": lambda: HullWhiteModel1F(
            0.1, 0.01, lambda t: 0.01 * torch.ones_like(t)).sample_paths([1.0], num_samples=4, **stateless),
        "GaussianHJM.sample_paths": lambda: GaussianHJM(1, [0.03], [0.01], flat).sample_paths(
            [1.0], 4, time_step=0.5, **stateless),
        "heston_european_mc": lambda: heston_european_mc(
            strikes=np.array([100.0]), expiry=1.0, spot=100.0, variance=0.04, mean_reversion=2.0, theta=0.04,
            volvol=0.3, rho=-0.7, discount_rate=0.02, num_samples=16, num_time_steps=4),
        "basket_european_mc": lambda: basket_european_mc(
            spots=np.full(2, 100.0), vols=np.array([0.2, 0.3]), rate=0.02, corr=np.eye(2), strike=100.0,
            expiry=1.0, num_time_steps=4, num_samples=16),
    }


@pytest.mark.parametrize("name", sorted(_calls()))
def test_public_call_raises_without_a_cuda_device(name):
    with pytest.raises(RuntimeError, match="CUDA device"):
        _calls()[name]()


def test_missing_library_raises_at_load():
    code = ("import sys; sys.path[:0] = [{root!r}, {pkg!r}]\n"
            "import tqf._lib as L\n"
            "L.LIB_PATH = '/nonexistent/libtqf.so'\n"
            "L._lib = None\n"
            "try:\n"
            "    L.load()\n"
            "except ImportError as e:\n"
            "    print('raised', e)\n").format(root=ROOT, pkg=os.path.join(ROOT, "tf-quant-finance_gb300"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.startswith("raised libtqf.so not found"), out.stdout
