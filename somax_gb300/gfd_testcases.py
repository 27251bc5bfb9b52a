"""Ready-made (model, state0) pairs of somax's test cases for the models this package runs
(``somax/_src/models/gfd_testcases.py``), with the same names, keyword arguments and defaults.

Each factory returns the GPU model and its initial state as float32 tensors on ``device``
(default: the current CUDA device); any extra keyword (``precision``, ``refine``, ...) goes to
the model's ``create``.
"""

from __future__ import annotations

import math

import torch

from .qg import BaroclinicQG, BaroclinicQGState, BarotropicQG, BarotropicQGState
from .reparameterized import MultilayerSW2DState, ReparameterizedQG
from .swm import MultilayerShallowWater2D, NonlinearShallowWater2D, NonlinearSW2DState


def _device(device):
    if device is not None:
        return torch.device(device)
    return torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu")


def barotropic_jet_instability(nx: int = 128, ny: int = 128, Lx: float = 1e6, Ly: float = 1e6, f0: float = 1e-4,
                               beta: float = 1.6e-11, H0: float = 1000.0, jet_speed: float = 1.0,
                               jet_width: float = 5e4, perturbation: float = 0.01, lateral_viscosity: float = 100.0,
                               device=None, **model_kw):
    """A Gaussian zonal jet with a sin(4 pi x / Lx) perturbation in a periodic single-layer
    basin (gfd_testcases.py:121-181)."""
    model = NonlinearShallowWater2D.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=f0, beta=beta, H0=H0,
                                           lateral_viscosity=lateral_viscosity, bc="periodic", **model_kw)
    g = model.grid
    u0, v0 = jet_fields(g.Nx, g.Ny, g.dx, g.dy, Lx, Ly, jet_speed, jet_width, perturbation, (1.0,))
    dev = _device(device)
    h0 = torch.full((g.Ny, g.Nx), float(H0), dtype=torch.float32, device=dev)
    return model, NonlinearSW2DState(h=h0, u=u0[0].to(device=dev, dtype=torch.float32),
                                     v=v0[0].to(device=dev, dtype=torch.float32))


def doublegyre_qg(nx: int = 64, ny: int = 64, Lx: float = 1e6, Ly: float = 1e6, f0: float = 1e-4,
                  beta: float = 1.6e-11, lateral_viscosity: float = 500.0, bottom_drag: float = 1e-7,
                  wind_amplitude: float = 1e-12, device=None, **model_kw):
    """Wind-driven barotropic double gyre from rest (gfd_testcases.py:184-228)."""
    model = BarotropicQG.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=f0, beta=beta, lateral_viscosity=lateral_viscosity,
                                bottom_drag=bottom_drag, wind_amplitude=wind_amplitude, wind_profile="doublegyre",
                                **model_kw)
    q0 = torch.zeros((model.grid.Ny, model.grid.Nx), dtype=torch.float32, device=_device(device))
    return model, BarotropicQGState(q=q0)


def doublegyre_baroclinic_qg(nx: int = 128, ny: int = 128, Lx: float = 4e6, Ly: float = 4e6, f0: float = 9.375e-5,
                             beta: float = 1.754e-11, n_layers: int = 3, H=(400.0, 1100.0, 2600.0),
                             g_prime=(9.81, 0.025, 0.0125), lateral_viscosity: float = 15.0,
                             bottom_drag: float = 1e-7, wind_amplitude: float = 1.3e-10, device=None, **model_kw):
    """Wind-driven multilayer double gyre from rest (gfd_testcases.py:231-287)."""
    model = BaroclinicQG.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=f0, beta=beta, n_layers=n_layers, H=H,
                                g_prime=g_prime, lateral_viscosity=lateral_viscosity, bottom_drag=bottom_drag,
                                wind_amplitude=wind_amplitude, wind_profile="doublegyre", **model_kw)
    q0 = torch.zeros((model.consts.n_layers, model.grid.Ny, model.grid.Nx), dtype=torch.float32,
                     device=_device(device))
    return model, BaroclinicQGState(q=q0)


def jet_fields(Nx: int, Ny: int, dx: float, dy: float, Lx: float, Ly: float, jet_speed: float, jet_width: float,
               perturbation: float, signs):
    """(u0, v0) of a layered jet in float64 on the host: a Gaussian zonal jet about y = Ly / 2
    with the given sign per layer and a sin(4 pi x / Lx) meridional perturbation under the same
    envelope, on every point of the padded grid (x_i = i dx, y_j = j dy)."""
    x = torch.arange(Nx, dtype=torch.float64) * dx
    y = torch.arange(Ny, dtype=torch.float64) * dy
    Y, X = torch.meshgrid(y, x, indexing="ij")
    env = torch.exp(-0.5 * ((Y - Ly / 2.0) / jet_width) ** 2)
    s = torch.tensor(signs, dtype=torch.float64)[:, None, None]
    u0 = s * jet_speed * env[None]
    v0 = (perturbation * torch.sin(4.0 * math.pi * X / Lx) * env)[None].expand(len(signs), Ny, Nx).clone()
    return u0, v0


def baroclinic_instability_swm(nx: int = 64, ny: int = 64, Lx: float = 1e6, Ly: float = 1e6, f0: float = 1e-4,
                               beta: float = 1.6e-11, H=(500.0, 4500.0), g_prime=(9.81, 0.025),
                               lateral_viscosity: float = 100.0, bottom_drag: float = 1e-7, jet_speed: float = 0.5,
                               jet_width: float = 5e4, perturbation: float = 0.01, device=None):
    """Two opposite zonal jets in a periodic 2-layer shallow-water basin
    (gfd_testcases.py:290-362): h at rest thickness, u the jet, v the perturbation."""
    nl = 2
    model = MultilayerShallowWater2D.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=f0, beta=beta, n_layers=nl, H=H,
                                            g_prime=g_prime, lateral_viscosity=lateral_viscosity,
                                            bottom_drag=bottom_drag, bc="periodic")
    g = model.grid
    u0, v0 = jet_fields(g.Nx, g.Ny, g.dx, g.dy, Lx, Ly, jet_speed, jet_width, perturbation, (1.0, -1.0)[:nl])
    Hs = torch.tensor([float(x) for x in model.strat.H], dtype=torch.float64)
    h0 = Hs[:, None, None].expand(nl, g.Ny, g.Nx).clone()
    dev = _device(device)
    return model, MultilayerSW2DState(*(t.to(device=dev, dtype=torch.float32) for t in (h0, u0, v0)))


def doublegyre_reparameterized_qg(nx: int = 128, ny: int = 128, Lx: float = 4e6, Ly: float = 4e6,
                                  f0: float = 9.375e-5, beta: float = 1.754e-11, n_layers: int = 3,
                                  H=(400.0, 1100.0, 2600.0), g_prime=(9.81, 0.025, 0.0125),
                                  lateral_viscosity: float = 15.0, bottom_drag: float = 3.6e-8,
                                  wind_amplitude: float = 8e-5, device=None, **model_kw):
    """Wind-driven double gyre of the reparameterised QG model in (h, u, v) from rest, wall
    boundaries (gfd_testcases.py:365-428)."""
    model = ReparameterizedQG.create(nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=f0, beta=beta, n_layers=n_layers, H=H,
                                     g_prime=g_prime, lateral_viscosity=lateral_viscosity, bottom_drag=bottom_drag,
                                     wind_amplitude=wind_amplitude, wind_profile="doublegyre", bc="wall", **model_kw)
    nl = model.consts.n_layers
    Ny, Nx = model.grid.Ny, model.grid.Nx
    dev = _device(device)
    Hs = torch.tensor([float(x) for x in model.strat.H], dtype=torch.float32)
    h0 = Hs[:, None, None].expand(nl, Ny, Nx).to(dev).contiguous()
    z = torch.zeros((nl, Ny, Nx), dtype=torch.float32, device=dev)
    return model, MultilayerSW2DState(h=h0, u=z, v=z.clone())


__all__ = ["barotropic_jet_instability", "doublegyre_qg", "doublegyre_baroclinic_qg", "baroclinic_instability_swm",
           "doublegyre_reparameterized_qg"]
