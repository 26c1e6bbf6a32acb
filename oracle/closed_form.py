"""Closed-form prices used to check Monte Carlo results.

* Black–Scholes (tff/black_scholes/vanilla_prices.py:28), SciPy ndtr.
* Heston European call/put by Fourier inversion of the characteristic
  function (the quantity tff/models/heston/approximations/european_option.py:30
  computes with Attari's formula and Simpson integration); here the
  Lewis/Gatheral "little Heston trap" form with adaptive quadrature.
"""

from __future__ import annotations

import numpy as np
from scipy import integrate
from scipy.special import ndtr


def black_scholes(spot, strike, rate, vol, expiry, is_call=True, dividend=0.0):
    spot, strike = np.asarray(spot, float), np.asarray(strike, float)
    fwd = spot * np.exp((rate - dividend) * expiry)
    sd = vol * np.sqrt(expiry)
    d1 = (np.log(fwd / strike) + 0.5 * sd * sd) / sd
    d2 = d1 - sd
    df = np.exp(-rate * expiry)
    call = df * (fwd * ndtr(d1) - strike * ndtr(d2))
    return np.where(is_call, call, call - df * (fwd - strike))


def _heston_cf(u, t, v0, kappa, theta, xi, rho):
    """E[exp(i u log(F_T/F_0))] under the forward measure (trap-free form)."""
    iu = 1j * u
    d = np.sqrt((rho * xi * iu - kappa) ** 2 + xi ** 2 * (iu + u * u))
    g = (kappa - rho * xi * iu - d) / (kappa - rho * xi * iu + d)
    e = np.exp(-d * t)
    C = kappa * theta / xi ** 2 * ((kappa - rho * xi * iu - d) * t - 2 * np.log((1 - g * e) / (1 - g)))
    D = (kappa - rho * xi * iu - d) / xi ** 2 * ((1 - e) / (1 - g * e))
    return np.exp(C + D * v0)


def heston_price(spot=None, forward=None, strike=100.0, expiry=1.0, rate=0.0, v0=0.04, kappa=2.0,
                 theta=0.04, xi=0.3, rho=-0.7, is_call=True, discount_factor=None):
    if forward is None:
        forward = spot * np.exp(rate * expiry)
    df = np.exp(-rate * expiry) if discount_factor is None else discount_factor
    k = np.log(strike / forward)

    def integrand(u, j):
        if j == 1:
            phi = _heston_cf(u - 1j, expiry, v0, kappa, theta, xi, rho) / _heston_cf(-1j, expiry, v0, kappa, theta, xi, rho)
        else:
            phi = _heston_cf(u, expiry, v0, kappa, theta, xi, rho)
        return (np.exp(-1j * u * k) * phi / (1j * u)).real

    p1 = 0.5 + integrate.quad(integrand, 1e-12, 400, args=(1,), limit=800, epsabs=1e-12)[0] / np.pi
    p2 = 0.5 + integrate.quad(integrand, 1e-12, 400, args=(2,), limit=800, epsabs=1e-12)[0] / np.pi
    call = df * (forward * p1 - strike * p2)
    if is_call:
        return call
    return call - df * (forward - strike)
