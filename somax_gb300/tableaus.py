"""Butcher tableaus of the explicit schemes integrate() accepts (diffrax equivalents)."""

from __future__ import annotations

# Tsitouras (2011) 5(4) pair, the coefficients of diffrax.Tsit5 (published values).
_TSIT5_A = [
    [],
    [0.161],
    [-0.008480655492356989, 0.335480655492357],
    [2.897153057105493, -6.359448489975075, 4.3622954328695815],
    [5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525],
    [5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383],
]
_TSIT5_B = [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
            2.324710524099774]


def rk_tableau(scheme: str):
    """(a, b) with a[s] the stage-s coefficients of the earlier stages."""
    if scheme == "euler":
        return [[]], [1.0]
    if scheme == "heun":
        return [[], [1.0]], [0.5, 0.5]
    if scheme == "ssprk3":
        return [[], [1.0], [0.25, 0.25]], [1 / 6, 1 / 6, 2 / 3]
    if scheme == "tsit5":
        return _TSIT5_A, _TSIT5_B
    raise ValueError(f"unknown scheme {scheme!r}")
