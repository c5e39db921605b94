"""Synthetic workloads (meshes + initial conditions) of the benchmark configurations.

No dataset is involved: every case is generated from seeded formulas.

* ``vortex_2d``: isentropic vortex on [-5, 5]^2, 32x32 Cartesian quads, row size 6,
  freestream Mach 0.5 along x, vortex strength 5 at the origin, Riemann-invariant
  freestream BCs on all faces. The state formula restates the reference's own vortex
  initial condition (include/Case.hil:69-82) with nondimensional peak velocity
  strength/(2 pi) and argmax radius 1, which is the classic strength-5 vortex.
* ``taylor_green_3d``: compressible Taylor-Green vortex on [0, 2 pi]^3, 32^3 deformed hexes
  whose interior vertices move by a seeded sinusoidal field of amplitude 0.1 element widths,
  row size 6, Mach 0.1, Re 1600, Pr 0.71, Sutherland viscosity and conductivity in SI
  units. hexed has no periodic BC, so the six faces use Nonpenetration walls, which are
  exact symmetry planes of the Taylor-Green flow at x, y, z in {0, 2 pi}.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .mesh import bc_spec, structured_mesh

HEAT_RAT = 1.4
R_AIR = 287.05287


def freestream_state(n_dim, mach, angle_deg=0., density=1.225, pressure=101325.):
    """Conserved freestream state [momentum..., density, energy]."""
    a = math.sqrt(HEAT_RAT * pressure / density)
    speed = mach * a
    vel = np.zeros(n_dim)
    vel[0] = speed * math.cos(math.radians(angle_deg))
    if n_dim > 1:
        vel[1] = speed * math.sin(math.radians(angle_deg))
    state = np.zeros(n_dim + 2)
    state[:n_dim] = density * vel
    state[n_dim] = density
    state[n_dim + 1] = pressure / (HEAT_RAT - 1) + 0.5 * density * speed * speed
    return state


def vortex_state(pos, fs, strength=5., radius=1., time=0.):
    """Isentropic vortex (include/Case.hil:69-82) around the origin.
    pos [2][...]; fs = freestream conserved state (2D)."""
    heat_rat = HEAT_RAT
    spec_int_ener = fs[3] / fs[2] - 0.5 * (fs[0] ** 2 + fs[1] ** 2) / fs[2] ** 2
    sound = (heat_rat * (heat_rat - 1) * spec_int_ener) ** 0.5
    nondim_veloc = strength / (2 * math.pi)
    x = pos[0] - fs[0] / fs[2] * time
    y = pos[1] - fs[1] / fs[2] * time
    gauss = nondim_veloc * np.exp((1. - (x ** 2 + y ** 2) / radius ** 2) / 2.)
    scalar = 1 - (heat_rat - 1.) / 2 * gauss ** 2
    mass = fs[2] * scalar ** (1. / (heat_rat - 1.))
    mom0 = (fs[0] / fs[2] - pos[1] / radius * gauss * sound) * mass
    mom1 = (fs[1] / fs[2] + pos[0] / radius * gauss * sound) * mass
    energy = spec_int_ener * scalar * mass + 0.5 * (mom0 ** 2 + mom1 ** 2) / mass
    return np.stack([mom0, mom1, mass, energy])


def vortex_2d(n_per_side=32, row_size=6, mach=0.5, strength=5.):
    """Config: 2D Euler isentropic vortex, Riemann-invariant freestream on all faces."""
    # nondimensional units: density 1, pressure 1/gamma (sound speed 1)
    fs = freestream_state(2, mach, density=1., pressure=1. / HEAT_RAT)
    spec = bc_spec(abi.BC_RIEMANN, freestream=fs)
    bcs = {(d, s): spec for d in range(2) for s in range(2)}
    ar = structured_mesh(2, row_size, n_per_side, -5., 5., bcs=bcs)
    ar.set_state(lambda pos: vortex_state(pos, fs, strength))
    ar.freestream = fs
    return ar


def tgv_transport(mach=0.1, reynolds=1600., prandtl=0.71, length=1., temperature=300.):
    """Dimensional set-up of the Taylor-Green case in SI units. Returns
    (rho0, v0, p0, visc, cond): the velocity scale v0 sets Mach 0.1 at the reference
    temperature; the density sets Re = rho v0 L / mu; Sutherland's law for air gives mu(T)
    and k(T) = mu(T) c_p / Pr with the same Sutherland offset (include/Transport_model.hpp:47-50)."""
    sound = math.sqrt(HEAT_RAT * R_AIR * temperature)
    v0 = mach * sound
    mu_ref, t_ref, offset = 1.716e-5, 273., 111.   # air (include/Case.hil:83-85)
    mu = mu_ref * (temperature / t_ref) ** 1.5 * (t_ref + offset) / (temperature + offset)
    rho0 = reynolds * mu / (v0 * length)
    p0 = rho0 * R_AIR * temperature
    cp = HEAT_RAT * R_AIR / (HEAT_RAT - 1)
    visc = abi.transport_sutherland(mu_ref, t_ref, offset)
    cond = abi.transport_sutherland(mu_ref * cp / prandtl, t_ref, offset)
    return rho0, v0, p0, visc, cond


def tgv_state(pos, rho0, v0, p0, length=1.):
    x, y, z = pos[0] / length, pos[1] / length, pos[2] / length
    u = v0 * np.sin(x) * np.cos(y) * np.cos(z)
    v = -v0 * np.cos(x) * np.sin(y) * np.cos(z)
    w = np.zeros_like(u)
    p = p0 + rho0 * v0 ** 2 / 16 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2)
    rho = rho0 * p / p0   # isothermal initial field
    e = p / (HEAT_RAT - 1) + 0.5 * rho * (u ** 2 + v ** 2 + w ** 2)
    return np.stack([rho * u, rho * v, rho * w, rho, e])


def sinusoid_displacement(h, amplitude=0.1, seed=0, n_dim=3):
    """Smooth vertex displacement of `amplitude` element widths, zero on the boundary."""
    rng = np.random.default_rng(seed)
    phase = rng.uniform(0, 2 * math.pi, size=(n_dim, n_dim))
    freq = rng.integers(1, 4, size=(n_dim, n_dim))

    def disp(pos, on_boundary):
        out = np.zeros_like(pos)
        for i in range(n_dim):
            f = np.ones(pos.shape[0])
            for j in range(n_dim):
                f = f * np.sin(freq[i, j] * pos[:, j] + phase[i, j])
            out[:, i] = amplitude * h * f
        out[on_boundary.any(axis=1)] = 0.
        return out
    return disp


def sphere_refinement(n_base, radius=0.25, centre=0.5):
    """Refinement predicate: cells of [0,1]^nd intersecting the sphere."""
    def refine(level, idx):
        h = 1.0 / (n_base * 2 ** level)
        lo = np.array(idx) * h
        p = np.clip(centre, lo, lo + h)
        return float(np.linalg.norm(p - centre)) <= radius
    return refine


def pulse_state(pos, fs, amplitude, width, centre):
    """Freestream plus a Gaussian pressure pulse of `amplitude` times the freestream pressure."""
    nd = pos.shape[0]
    rho, mom = fs[nd], fs[:nd]
    p_inf = (HEAT_RAT - 1) * (fs[nd + 1] - 0.5 * float(mom @ mom) / rho)
    r2 = sum((pos[d] - centre[d]) ** 2 for d in range(nd))
    p = p_inf * (1 + amplitude * np.exp(-r2 / width ** 2))
    st = [np.full_like(pos[0], m) for m in mom] + [np.full_like(pos[0], rho)]
    st.append(p / (HEAT_RAT - 1) + 0.5 * float(mom @ mom) / rho)
    return np.stack(st)


def pulse_tree_3d(n_base=16, row_size=4, levels=2, mach=0.3, seed=0, amplitude=0.01, width=0.05):
    """Config: 3D adapted mesh with hanging faces. 16^3 base hexes on [0,1]^3 refined
    `levels` times in every cell intersecting a centred sphere of radius 0.25 (2:1
    balanced), Euler at Mach 0.3 with a Gaussian pressure pulse (amplitude 0.01 p_inf,
    width 0.05) at a seeded random point; Riemann-invariant freestream on the faces."""
    from .tree import tree_mesh
    rng = np.random.default_rng(seed)
    centre = rng.uniform(0.3, 0.7, size=3)
    fs = freestream_state(3, mach, 0., 1.2, 1e5)
    spec = bc_spec(abi.BC_RIEMANN, freestream=fs)
    ar = tree_mesh(3, row_size, n_base, levels, sphere_refinement(n_base),
                   {(d, s): spec for d in range(3) for s in range(2)})
    ar.set_state(lambda pos: pulse_state(pos, fs, amplitude, width, centre))
    ar.freestream = fs
    ar.pulse_centre = centre
    return ar


def mach2_jump_3d(n_per_side=32, row_size=6, seed=0, amplitude=0.1, density_ratio=2.5, mach=2.):
    """Config: the deformed 32^3 mesh of the Taylor-Green case carrying an inviscid Mach 2
    flow along x with a planar density jump (ratio 2.5, equal pressure) at x = pi, which the
    stabilising artificial viscosity (Solver::set_art_visc_admis) must act on. Riemann-
    invariant freestream on the x faces, Nonpenetration on the faces parallel to the flow.
    `av_char_speed` is the freestream speed plus sound speed (src/Solver.cpp:640)."""
    length = 2 * math.pi
    h = length / n_per_side
    fs = freestream_state(3, mach, 0., 1.2, 1e5)
    riemann = bc_spec(abi.BC_RIEMANN, freestream=fs)
    wall = bc_spec(abi.BC_NONPENETRATION)
    bcs = {(d, s): (riemann if d == 0 else wall) for d in range(3) for s in range(2)}
    ar = structured_mesh(3, row_size, n_per_side, 0., length, deformed=True,
                         displacement=sinusoid_displacement(h, amplitude, seed), bcs=bcs)

    def state(pos):
        rho = np.where(pos[0] < math.pi, 1.2, 1.2 * density_ratio)
        vel = fs[0] / fs[3]
        p = 1e5
        return np.stack([rho * vel, 0 * rho, 0 * rho, rho, p / (HEAT_RAT - 1) + 0.5 * rho * vel * vel])
    ar.set_state(state)
    ar.freestream = fs
    sound = math.sqrt(HEAT_RAT * 1e5 / 1.2)
    ar.av_char_speed = mach * sound + sound
    return ar


def taylor_green_3d(n_per_side=32, row_size=6, mach=0.1, reynolds=1600., seed=0, amplitude=0.1):
    """Config: 3D compressible Navier-Stokes Taylor-Green vortex on deformed hexes."""
    length = 2 * math.pi
    rho0, v0, p0, visc, cond = tgv_transport(mach, reynolds)
    h = length / n_per_side
    spec = bc_spec(abi.BC_NONPENETRATION)
    bcs = {(d, s): spec for d in range(3) for s in range(2)}
    ar = structured_mesh(3, row_size, n_per_side, 0., length, deformed=True,
                         displacement=sinusoid_displacement(h, amplitude, seed), bcs=bcs)
    ar.set_state(lambda pos: tgv_state(pos, rho0, v0, p0))
    ar.visc, ar.cond = visc, cond
    ar.seed = seed
    return ar
