"""Linear potential-flow problems and results (problems_and_results.jl:1-227)."""
from __future__ import annotations

import math

import numpy as np

SETTINGS = {"rho": 1000.0, "g": 9.81}  # constants.jl:10-29


def set_g(val: float):
    SETTINGS["g"] = float(val)


def set_rho(val: float):
    SETTINGS["rho"] = float(val)


def compute_wavenumber(omega, g=None):
    """Deep-water dispersion k = omega^2 / g (waves.jl:133-134)."""
    g = SETTINGS["g"] if g is None else g
    return omega * omega / g


def compute_encountered_values(omega, beta, forward_speed, g=None):
    """compute_encountered_values (waves.jl:136-151) -> (omega_e, k_e, beta_e)."""
    g = SETTINGS["g"] if g is None else g
    k = compute_wavenumber(omega, g)
    if forward_speed == 0:
        return omega, k, beta
    doppler = omega - k * forward_speed * math.cos(beta)
    oe = abs(doppler)
    ke = compute_wavenumber(oe, g)
    be = beta if doppler >= 0 else beta + math.pi
    return oe, ke, be


class LinearPotentialFlowProblem:
    def _common(self, body, omega, beta, wavenumber, forward_speed, influenced_dofs, rho, g):
        self.floatingbody = body
        self.rho = SETTINGS["rho"] if rho is None else float(rho)
        self.g = SETTINGS["g"] if g is None else float(g)
        self.omega = float(omega)
        self.beta = 0.0 if beta is None else float(beta)
        self.wavenumber = compute_wavenumber(self.omega, self.g) if wavenumber is None else float(wavenumber)
        self.forward_speed = float(forward_speed)
        inf = list(body.dofs) if influenced_dofs is None else [str(d) for d in influenced_dofs]
        for d in inf:
            if d not in body.dofs:
                raise ValueError("each influenced_dofs name must be a key of floatingbody.dofs")
        self.influenced_dofs = inf
        if self.forward_speed == 0:
            self.encountered_omega, self.encountered_wavenumber, self.encountered_beta = (
                self.omega, self.wavenumber, self.beta)
        else:
            self.encountered_omega, self.encountered_wavenumber, self.encountered_beta = compute_encountered_values(
                self.omega, self.beta, self.forward_speed, self.g)


class RadiationProblem(LinearPotentialFlowProblem):
    """RadiationProblem (problems_and_results.jl:84-150)."""

    def __init__(self, body, omega, radiating_dof=None, influenced_dofs=None, beta=None, forward_speed=0.0,
                 wavenumber=None, rho=None, g=None):
        self._common(body, omega, beta, wavenumber, forward_speed, influenced_dofs, rho, g)
        if radiating_dof is None:
            if len(self.influenced_dofs) != 1:
                raise ValueError("radiating_dof is required when there is more than one influenced dof")
            radiating_dof = self.influenced_dofs[0]
        if str(radiating_dof) not in body.dofs:
            raise ValueError("the radiating_dof must be a key of floatingbody.dofs")
        self.radiating_dof = str(radiating_dof)


class DiffractionProblem(LinearPotentialFlowProblem):
    """DiffractionProblem (problems_and_results.jl:14-78)."""

    def __init__(self, body, omega, beta=0.0, influenced_dofs=None, forward_speed=0.0, wavenumber=None, rho=None,
                 g=None):
        self._common(body, omega, beta, wavenumber, forward_speed, influenced_dofs, rho, g)


def remake(prob, **kw):
    """remake (problems_and_results.jl:152-185)."""
    body = kw.get("floatingbody", prob.floatingbody)
    omega = kw.get("omega", prob.omega)
    g = kw.get("g", prob.g)
    rho = kw.get("rho", prob.rho)
    fs = kw.get("forward_speed", prob.forward_speed)
    inf = kw.get("influenced_dofs", prob.influenced_dofs)
    k = kw["wavenumber"] if "wavenumber" in kw else (compute_wavenumber(omega, g) if "omega" in kw else prob.wavenumber)
    if isinstance(prob, RadiationProblem):
        return RadiationProblem(body, omega, kw.get("radiating_dof", prob.radiating_dof), inf,
                                kw.get("beta", prob.beta if fs != 0 else None), fs, k, rho, g)
    return DiffractionProblem(body, omega, kw.get("beta", prob.beta), inf, fs, k, rho, g)


class RadiationResult:
    def __init__(self, problem, forces: dict):
        self.problem = problem
        self.forces = forces


class DiffractionResult:
    def __init__(self, problem, forces: dict):
        self.problem = problem
        self.forces = forces


def _result_omega(res):
    p = res.problem
    return p.omega if p.forward_speed == 0 else p.encountered_omega


def added_mass(res: RadiationResult) -> dict:
    """A = Re(F)/omega^2 (problems_and_results.jl:207)."""
    w = _result_omega(res)
    return {k: v.real / w ** 2 for k, v in res.forces.items()}


def radiation_damping(res: RadiationResult) -> dict:
    """B = Im(F)/omega (problems_and_results.jl:208)."""
    w = _result_omega(res)
    return {k: v.imag / w for k, v in res.forces.items()}


def radiation_coefficients(res: RadiationResult) -> dict:
    return {"added_mass": added_mass(res), "radiation_damping": radiation_damping(res)}


def diffraction_force(res: DiffractionResult) -> dict:
    return dict(res.forces)


def make_result(problem, forces):
    return RadiationResult(problem, forces) if isinstance(problem, RadiationProblem) else DiffractionResult(problem,
                                                                                                             forces)
