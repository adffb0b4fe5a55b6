"""Pole algebra with the reference's API and evaluation semantics
(pyhub/tools/pole.py:5-197): G(w) = sum_k weights_k / (w - positions_k + i eta).

Evaluation is vectorised with numpy instead of the reference's per-pole
Python loops; results agree to rounding (tests/golden holds vectors produced
by the reference's own module).
"""
from __future__ import annotations

from typing import Callable

import numpy as np


class Pole:
    r"""A set of poles given by {'positions': [...], 'weights': [...]}."""

    def __init__(self, pole: dict, atol=1.e-10):
        # the reference accepts exactly this key order (pole.py:10)
        if list(pole.keys()) != ['positions', 'weights']:
            raise ValueError(f"Pole asked is not correct, use correct notation -> "
                             f"{str({'positions': [], 'weights': []})} not {pole.keys()}")
        self.pole = {'positions': np.array(pole['positions'], copy=True, dtype=float),
                     'weights': np.array(pole['weights'], copy=True, dtype=float)}
        self.atol = atol
        if len(pole['weights']) != len(pole['positions']):
            raise ValueError(f"number of poles {len(pole['positions'])} should be equal as len of weights "
                             f"{len(pole['weights'])}")

    def __call__(self, w, eta: float = 0.05):
        return self.retarded(w, eta=eta)

    def __str__(self):
        return f"{self.pole}"

    def __add__(self, other):
        return Pole({'positions': np.concatenate((self.pole['positions'], other.pole['positions'])),
                     'weights': np.concatenate((self.pole['weights'], other.pole['weights']))})

    def __sub__(self, other):
        return Pole({'positions': np.concatenate((self.pole['positions'], other.pole['positions'])),
                     'weights': np.concatenate((self.pole['weights'], -other.pole['weights']))})

    def __mul__(self, other):
        if isinstance(other, (float, int, complex, np.complex128, np.floating)):
            return Pole({'positions': self.pole['positions'], 'weights': self.pole['weights'] * other})
        raise TypeError(f"Other must be float complex or int, not {type(other)}")

    def __truediv__(self, other):
        if isinstance(other, (float, int, np.floating)):
            return Pole({'positions': self.pole['positions'], 'weights': self.pole['weights'] / other})
        raise TypeError(f"Other must be float or int, not {type(other)}")

    def shift(self, s: float):
        return Pole({'positions': s + self.pole['positions'], 'weights': self.pole['weights']})

    def clean(self, ptol=1.e-5, wtol=1.e-5):
        """Drop |weight| < wtol, then merge positions equal after rounding to
        int(-log10(ptol)) decimals (pole.py:69-78)."""
        index = np.where(abs(self.pole['weights']) < wtol)[0]
        self.pole['weights'] = np.delete(self.pole['weights'], index)
        self.pole['positions'] = np.delete(self.pole['positions'], index)
        self.pole['positions'], index = np.unique(np.around(self.pole['positions'], int(-np.log10(ptol))),
                                                  return_inverse=True)
        new_weights = np.zeros(self.nb_poles)
        np.add.at(new_weights, index, self.pole['weights'])
        self.pole['weights'] = new_weights
        return self

    def _eval(self, w, shift):
        p, wt = self.pole['positions'], self.pole['weights']
        if isinstance(w, (float, complex, int, np.floating, np.complexfloating)):
            return complex(np.sum(wt / (w - p + shift)))
        w = np.asarray(w)
        return (wt[None, :] / (w[:, None] - p[None, :] + shift)).sum(axis=1)

    def retarded(self, w, eta: float = 0.05) -> complex:
        return self._eval(w, 1j * eta)

    def advanced(self, w, eta: float = 0.05) -> complex:
        return self._eval(w, -1j * eta)

    def greater(self, w, ef, eta: float = 0.05) -> complex:
        sel = self.pole['positions'] > ef
        return Pole({'positions': self.pole['positions'][sel], 'weights': self.pole['weights'][sel]})._eval(w, -1j * eta)

    def lesser(self, w, ef, eta: float = 0.05) -> complex:
        sel = self.pole['positions'] < ef
        return Pole({'positions': self.pole['positions'][sel], 'weights': self.pole['weights'][sel]})._eval(w, 1j * eta)

    def causal(self, w, ef, eta: float = 0.05) -> complex:
        p, wt = self.pole['positions'], self.pole['weights']
        s = np.sign(p - ef) * 1j * eta
        if isinstance(w, (float, complex, int, np.floating)):
            return complex(np.sum(wt / (w - p + s)))
        w = np.asarray(w)
        return (wt[None, :] / (w[:, None] - p[None, :] + s[None, :])).sum(axis=1)

    def spectral_density(self, w, eta: float = 0.05):
        return -1. * np.imag(self.retarded(w, eta)) / np.pi

    @classmethod
    def empty(cls):
        return cls({'positions': np.array([]), 'weights': np.array([])})

    @classmethod
    def zero(cls):
        return cls({'positions': np.array([0.]), 'weights': np.array([0.])})

    @classmethod
    def pole_research(cls, gf: Callable[[float], complex], borne: np.ndarray, eta: float = 0.01, crit: float = 1.,
                      eta_is_var: bool = True, constant=True):
        """Lorentzian peak search on a grid (pole.py:112-146)."""
        from scipy.optimize import minimize_scalar as ms
        low, nb_steps, dw = borne[0], len(borne), np.average(borne[1:] - borne[:-1])
        pole = {'positions': np.array([]), 'weights': np.array([])}
        elem_list = [-gf(low - dw, eta=eta).imag, -gf(low, eta=eta).imag]
        new_eta = eta / 10 if eta_is_var else eta
        for k in range(nb_steps):
            elem_list.append(-gf(low + (k + 1) * dw, eta=eta).imag)
            if abs(elem_list[1]) >= crit * abs(elem_list[0]) and abs(elem_list[1]) >= crit * abs(elem_list[2]):
                w_max = ms(lambda w: -abs(gf(w, eta=new_eta).imag),
                           bounds=(low + (k - 1) * dw, low + (k + 1) * dw), method='bounded').x
                pole['positions'] = np.append(pole['positions'], w_max)
                pole['weights'] = np.append(pole['weights'], -gf(w_max, eta=new_eta).imag * new_eta)
            del elem_list[0]
        if constant and abs(gf(1.e5, eta=eta).real) >= 1 / 1.e4:
            pole['positions'] = np.append(pole['positions'], 1.e8)
            pole['weights'] = np.append(pole['weights'], -(1.e8) * gf(1.e5, eta=eta).real)
        return cls(pole)

    @staticmethod
    def sum(l):
        pos = [p.pole['positions'] for p in l]
        wts = [p.pole['weights'] for p in l]
        if not pos:
            return Pole.empty()
        return Pole({'positions': np.concatenate(pos), 'weights': np.concatenate(wts)})

    @property
    def nb_poles(self):
        return len(self.pole['positions'])
