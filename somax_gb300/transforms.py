"""Stratification profiles and layer <-> mode transforms (host-side set-up, float64).

Mirrors ``somax/_src/core/transforms.py`` (``StratificationProfile`` :11-148,
``ModalTransform`` :151-224).  The coupling matrix A is the layered-QG stretching operator
(finitevolx ``build_coupling_matrix``, called at transforms.py:192); the modes are its right
eigenvectors sorted by ascending eigenvalue, Cl2m = Cm2l^-1.
"""

from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class StratificationProfile:
    """Layer thicknesses H (top to bottom), reduced gravities g_prime, optional densities."""

    H: np.ndarray
    g_prime: np.ndarray
    rho: np.ndarray | None = None

    @property
    def nl(self) -> int:
        return int(self.H.shape[0])

    @property
    def total_depth(self) -> float:
        return float(np.sum(self.H))

    @staticmethod
    def from_N2_constant(N2: float, depth: float, n_layers: int, g: float = 9.81, rho0: float = 1025.0):
        """transforms.py:41-76: equal layers, g'[0] = g, g'[k >= 1] = N2 * H_k."""
        Hk = depth / n_layers
        H = np.full(n_layers, Hk)
        gp = np.concatenate([[g], np.full(n_layers - 1, N2 * Hk)])
        rho = rho0 + rho0 * N2 * Hk / g * np.arange(n_layers)
        return StratificationProfile(H=H, g_prime=gp, rho=rho)

    @staticmethod
    def from_N2_exponential(N2_surface: float, scale_depth: float, depth: float, n_layers: int,
                            g: float = 9.81, rho0: float = 1025.0):
        """transforms.py:78-115."""
        Hk = depth / n_layers
        H = np.full(n_layers, Hk)
        z_if = -np.arange(1, n_layers) * Hk
        gp = np.concatenate([[g], N2_surface * np.exp(z_if / scale_depth) * Hk])
        z_c = -(np.arange(n_layers) + 0.5) * Hk
        rho = rho0 + np.cumsum(rho0 * N2_surface * np.exp(z_c / scale_depth) * Hk / g)
        return StratificationProfile(H=H, g_prime=gp, rho=rho)

    @staticmethod
    def from_layers(H, g_prime, rho=None):
        """transforms.py:117-148."""
        if len(H) != len(g_prime):
            raise ValueError(f"H ({len(H)}) and g_prime ({len(g_prime)}) must have the same length")
        if rho is not None and len(rho) != len(H):
            raise ValueError(f"rho ({len(rho)}) must have the same length as H ({len(H)})")
        return StratificationProfile(H=np.asarray(H, float), g_prime=np.asarray(g_prime, float),
                                     rho=None if rho is None else np.asarray(rho, float))


def coupling_matrix(H, g_prime) -> np.ndarray:
    """Tridiagonal stretching operator A: (A psi)_k couples layer k to k-1 through g'[k]
    and to k+1 through g'[k+1]; the top interface uses g'[0]."""
    H = np.asarray(H, float)
    g = np.asarray(g_prime, float)
    n = H.size
    A = np.zeros((n, n))
    for k in range(n):
        up = 1.0 / g[k]  # interface above layer k
        dn = 1.0 / g[k + 1] if k + 1 < n else 0.0  # interface below (none for the bottom)
        A[k, k] = (up + dn) / H[k]
        if k > 0:
            A[k, k - 1] = -up / H[k]
        if k + 1 < n:
            A[k, k + 1] = -dn / H[k]
    return A


@dataclasses.dataclass
class ModalTransform:
    """transforms.py:151-224.  ``eigs`` selects where the Helmholtz eigenvalues come from:
    "consistent" = eig(A) paired with the modes, "reference" = eigh of the symmetrised A as
    ``jnp.linalg.eigh`` computes at transforms.py:194."""

    Cl2m: np.ndarray
    Cm2l: np.ndarray
    eigenvalues: np.ndarray
    rossby_radii: np.ndarray

    @staticmethod
    def from_physics(H, g_prime, f0: float, eigs: str = "consistent") -> "ModalTransform":
        A = coupling_matrix(H, g_prime)
        lam, R = np.linalg.eig(A)
        order = np.argsort(lam.real)
        lam = lam.real[order]
        R = R.real[:, order]
        with np.errstate(divide="ignore", invalid="ignore"):
            radii = 1.0 / (f0 * np.sqrt(lam))
        if eigs == "consistent":
            ev = lam
        elif eigs == "reference":
            ev = np.linalg.eigvalsh(0.5 * (A + A.T))
        else:
            raise ValueError(f"unknown eigs mode {eigs!r}")
        return ModalTransform(Cl2m=np.linalg.inv(R), Cm2l=R, eigenvalues=ev, rossby_radii=radii)

    @staticmethod
    def from_stratification(strat: StratificationProfile, f0: float, eigs: str = "consistent"):
        return ModalTransform.from_physics(strat.H, strat.g_prime, f0, eigs)

    def to_modal(self, x):
        """Cl2m along the leading (layer) axis (transforms.py:218-220)."""
        return _apply_layers(self.Cl2m, x)

    def to_layer(self, x):
        """Cm2l along the leading (layer) axis (transforms.py:222-224)."""
        return _apply_layers(self.Cm2l, x)


def _apply_layers(M, x):
    try:
        import torch

        if isinstance(x, torch.Tensor):
            Mt = torch.as_tensor(M, dtype=x.dtype, device=x.device)
            return torch.einsum("lm,m...->l...", Mt, x)
    except ImportError:  # pragma: no cover
        pass
    return np.einsum("lm,m...->l...", M.astype(np.asarray(x).dtype), x)
