"""tff.math.qmc on the GPU: known answers of the reference's qmc tests and
parity with the oracle restatement (digital nets, scrambling, lattice rules)."""

import json
import os

import numpy as np
import pytest
import torch

from oracle import qmc as oqmc

pytestmark = pytest.mark.gpu


def _golden():
    with open(os.path.join(os.path.dirname(__file__), "golden", "qmc_golden.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_known_answers(cuda, dtype):
    from tqf.math import qmc
    g = _golden()
    tol = dict(rtol=1e-6, atol=1e-6)
    c = g["generating_matrices"]
    for idt in (torch.int32, torch.int64):
        m = qmc.sobol_generating_matrices(c["dim"], c["num_results"], c["num_digits"], validate_args=True, dtype=idt)
        assert m.dtype == idt
        np.testing.assert_array_equal(m.cpu().numpy(), c["expected"])
    for key in ("sobol_sample", "sobol_sample_indices", "sobol_sample_tent", "sobol_sample_dtype"):
        c = g[key]
        got = qmc.sobol_sample(c["dim"], c["num_results"], sequence_indices=c.get("sequence_indices"),
                               apply_tent_transform=c.get("tent", False), validate_args=True, dtype=dtype)
        assert got.dtype == dtype
        np.testing.assert_allclose(got.cpu().numpy(), c["expected"], **tol)
    for key in ("digital_net", "digital_net_indices", "digital_net_tent"):
        c = g[key]
        gen = qmc.sobol_generating_matrices(c["dim"], c["num_results"], c["num_digits"])
        got = qmc.digital_net_sample(gen, c["num_results"], c["num_digits"],
                                     sequence_indices=c.get("sequence_indices"),
                                     apply_tent_transform=c.get("tent", False), validate_args=True, dtype=dtype)
        np.testing.assert_allclose(got.cpu().numpy(), c["expected"], **tol)
    gv = torch.as_tensor(g["lattice_generating_vectors"], dtype=torch.int32)
    for key, shift in (("lattice", None), ("lattice_indices", None), ("lattice_zero_shift", torch.zeros(20)),
                       ("lattice_shift", g["lattice_shift"].get("additive_shift"))):
        c = g[key]
        got = qmc.lattice_rule_sample(gv, c["dim"], c["num_results"], sequence_indices=c.get("sequence_indices"),
                                      additive_shift=shift, validate_args=True, dtype=dtype)
        np.testing.assert_allclose(got.cpu().numpy(), c["expected"], **tol)


def test_scrambled_and_shifted_nets_match_oracle(cuda):
    from tqf.math import qmc
    dim, n = 12, 4096
    nd = int(np.ceil(np.log2(n)))
    smat = qmc.random_scrambling_matrices(dim, nd, seed=(2, 3))
    shift = qmc.random_digital_shift(dim, nd, seed=(4, 5))
    s = smat.cpu().numpy()
    assert s.shape == (dim, nd) and s.min() >= 2 ** (nd - 1) and s.max() < 2 ** nd
    assert np.array_equal(s, qmc.random_scrambling_matrices(dim, nd, seed=(2, 3)).cpu().numpy())
    got = qmc.sobol_sample(dim, n, scrambling_matrices=smat, digital_shift=shift, dtype=torch.float64)
    want = oqmc.sobol_sample(dim, n, scrambling_matrices=s, digital_shift=shift.cpu().numpy(), dtype=np.float64)
    np.testing.assert_array_equal(got.cpu().numpy(), want)
    # scrambling with the minimum matrices is the identity (digital_net_test.py:272-301)
    gen = qmc.sobol_generating_matrices(6, 8, 3)
    same = qmc.scramble_generating_matrices(gen, torch.full(gen.shape, 4, dtype=gen.dtype), 3)
    np.testing.assert_array_equal(same.cpu().numpy(), gen.cpu().numpy())
    v = qmc.random_scrambling_vectors(20, seed=(2, 3), validate_args=True)
    assert v.shape == (20,) and float(v.min()) >= 0 and float(v.max()) < 1
    # a scrambled net still integrates x1 x2 ... to 1/2^dim-ish accuracy
    pts = got.cpu().numpy()
    np.testing.assert_allclose(pts.mean(0), 0.5, atol=2e-3)
