"""Correlated GBM: drop-in for tff.models.MultivariateGeometricBrownianMotion
(tff/models/geometric_brownian_motion/multivariate_geometric_brownian_motion.py:40-281).

``sample_paths`` runs the reference's exact log scheme — per requested time
(time grid [0] + times), log increments (mu - sigma^2/2) dt + sqrt(dt) sigma
L z with L = chol(corr), cumulated and exponentiated — in
``tqf_mvgbm_paths``; the Cholesky factor is computed in FP64 on the GPU
(``tqf_cholesky_f64``).
"""

from __future__ import annotations

import numpy as np
import torch

from tqf import _lib
from tqf.math.random import multivariate_normal as mvn
from tqf.math.random.multivariate_normal import RandomType
from tqf.models import utils
from tqf.models.ito_process import ItoProcess


def cholesky_f64(corr, device) -> torch.Tensor:
    """FP64 lower Cholesky factor of a correlation matrix, on the device."""
    a = torch.as_tensor(utils.to_numpy(corr, np.float64)).to(device).contiguous()
    n = a.shape[0]
    L = torch.empty_like(a)
    info = torch.zeros(1, dtype=torch.int32, device=device)
    _lib.call("tqf_cholesky_f64", a.data_ptr(), n, L.data_ptr(), info.data_ptr(), _lib.stream_ptr(device))
    if int(info.item()) != 0:
        raise ValueError(f"correlation matrix is not positive definite (pivot {int(info.item()) - 1})")
    return L


class MultivariateGeometricBrownianMotion(ItoProcess):

    def __init__(self, dim, means=0.0, volatilities=1.0, corr_matrix=None, dtype=None, name=None):
        self._name = name or "multivariate_geometric_brownian_motion"
        self._dim = int(dim)
        np_dt = utils.np_dtype(dtype) if dtype is not None else utils.infer_dtype(means)
        self._np_dtype = np_dt
        self._means = np.broadcast_to(utils.to_numpy(means, np_dt), (self._dim,)).astype(np_dt)
        self._vols = np.broadcast_to(utils.to_numpy(volatilities, np_dt), (self._dim,)).astype(np_dt)
        if corr_matrix is None:
            self._corr = None
        else:
            self._corr = utils.to_numpy(corr_matrix, np_dt)
            if list(self._corr.shape) != [self._dim, self._dim]:
                raise ValueError("`corr_matrix` must be of shape [{0}, {0}] but is of shape {1}".format(
                    self._dim, list(self._corr.shape)))

    def dim(self):
        return self._dim

    def dtype(self):
        return utils.torch_dtype(self._np_dtype)

    def name(self):
        return self._name

    def drift_fn(self):
        """a(t, x) = means * x, in the process dtype
        (multivariate_geometric_brownian_motion.py:127-133)."""
        def _drift_fn(t, x):
            del t
            x = torch.as_tensor(x).to(self.dtype())
            return torch.as_tensor(self._means, device=x.device) * x
        return _drift_fn

    def volatility_fn(self):
        """b(t, x) = (volatilities * x)[:, None] * chol(corr_matrix), or
        diag(volatilities * x) without a correlation matrix (:135-150)."""
        def _vol_fn(t, x):
            del t
            x = torch.as_tensor(x).to(self.dtype())
            vols = torch.as_tensor(self._vols, device=x.device) * x
            if self._corr is None:
                return torch.diag_embed(vols)
            chol = torch.linalg.cholesky(torch.as_tensor(self._corr, dtype=torch.float64))
            return vols[..., None] * chol.to(dtype=vols.dtype, device=vols.device)
        return _vol_fn

    def sample_paths(self, times, initial_state=None, num_samples=1, random_type=None, seed=None, skip=0,
                     normal_draws=None, name=None, lz_mode=0):
        """Returns [num_samples, k, dim] (multivariate_geometric_brownian_motion.py:153-227).

        ``lz_mode`` (extension): 0 computes L z on the tensor cores (split BF16,
        three products) for 16 to 64 correlated float32 factors, 1 forces CUDA
        cores."""
        del name
        launch, out = self.paths_launcher(times, initial_state, num_samples, random_type, seed, skip,
                                          normal_draws, lz_mode)
        launch()
        return out

    def paths_launcher(self, times, initial_state=None, num_samples=1, random_type=None, seed=None, skip=0,
                       normal_draws=None, lz_mode=0):
        """Prepares one sample_paths launch: returns (launch, out), where
        launch() runs the path kernel into the preallocated ``out`` on the
        current stream (repeatable, for timing and graph capture)."""
        np_dt = self._np_dtype
        td = utils.torch_dtype(np_dt)
        times_np = utils.to_numpy(times, np_dt).reshape(-1)
        k = len(times_np)
        if normal_draws is not None and tuple(normal_draws.shape)[-1] != self._dim:
            raise ValueError("`dim` should be equal to `normal_draws.shape[2]` but are "
                             f"{self._dim} and {tuple(normal_draws.shape)[-1]} respectively")
        device = _lib.require_cuda()
        keep_alive = []
        if normal_draws is not None:
            dr = normal_draws if isinstance(normal_draws, torch.Tensor) else torch.as_tensor(
                utils.to_numpy(normal_draws, np_dt))
            dr = dr.to(device=device, dtype=td)
            keep_alive.append(dr)
            num_samples = int(dr.shape[0])
            draws = mvn.memory_draws(dr, path_axis=0, step_axis=1)
        else:
            rt = RandomType.PSEUDO if random_type is None else random_type
            if rt in (RandomType.SOBOL, RandomType.HALTON, RandomType.HALTON_RANDOMIZED):
                sob = utils.generate_mc_normal_draws(self._dim, k, int(num_samples), rt, skip=skip, seed=seed,
                                                     dtype=td)
                keep_alive.append(sob)
                draws = mvn.memory_draws(sob, path_axis=1, step_axis=0)
            else:
                draws = mvn.philox_draws(rt, seed, int(num_samples))
        N = int(num_samples)
        if initial_state is None:
            x0 = torch.ones(self._dim, dtype=td, device=device)
        else:
            x0 = torch.as_tensor(utils.to_numpy(initial_state, np_dt)).to(device)
            x0 = torch.broadcast_to(x0, (N, self._dim)).contiguous() if x0.dim() > 1 else x0.reshape(self._dim)
        grid = np.concatenate([[np_dt.type(0)], times_np]).astype(np_dt)
        dt = (grid[1:] - grid[:-1]).astype(np_dt)
        rows = np.zeros((k, 4), np.float64)
        rows[:, 0] = dt
        rows[:, 1] = np.sqrt(dt).astype(np_dt)
        rows[:, 2] = np.arange(k)
        table = utils.step_table(rows, td, device)
        drift = torch.as_tensor((self._means.astype(np.float64) - self._vols.astype(np.float64) ** 2 / 2)).to(device, td)
        vol = torch.as_tensor(self._vols).to(device)
        chol = cholesky_f64(self._corr, device).to(td) if self._corr is not None else None
        out = torch.empty((N, k, self._dim), dtype=td, device=device)
        a = _lib.MvgbmArgs()
        a.dtype = _lib.dtype_code(td)
        a.dim = self._dim
        a.num_paths = N
        a.num_steps = k
        a.x0_per_path = 1 if x0.dim() == 2 else 0
        a.step_table = table.data_ptr()
        a.x0 = x0.data_ptr()
        a.drift = drift.data_ptr()
        a.vol = vol.data_ptr()
        a.chol = chol.data_ptr() if chol is not None else None
        a.draws = draws
        a.output.ptr = out.data_ptr()
        a.output.num_slots = k
        a.output.init_slot = -1
        a.output.every_step = 1  # date j records slot j
        a.dev_status = _lib.status_buffer(device).data_ptr()
        a.lz_mode = int(lz_mode)  # 0: tensor cores for 16-64 float32 factors, 1: CUDA cores
        keep_alive += [x0, table, drift, vol, chol]

        def launch():
            _ = keep_alive
            _lib.call("tqf_mvgbm_paths", a, _lib.stream_ptr(device))

        return launch, out


__all__ = ["MultivariateGeometricBrownianMotion", "cholesky_f64"]
