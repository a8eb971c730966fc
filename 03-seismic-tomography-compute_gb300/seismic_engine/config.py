"""The reference's configuration types and YAML reader: SolverConfig /
ModelConfig / InversionConfig / TomographyConfig (core/config.h:9-51) and
load_config (core/config.cpp:9-94), restated line for line in behaviour:
hard-coded defaults, a two-level `section:` / `key: value` reader that
ignores indentation, comments, unknown sections and unknown keys, and parses
numbers like std::stod / std::stoi (leading numeric prefix; no number at all
raises). Keys the reference does not parse (seafloor_gradient,
snapshot_interval, output_dir, vs/rho bounds, misfit_tolerance,
gradient_precondition, line_search_*) keep their defaults, as there.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

from .wave import SolverConfig

_FLOAT = re.compile(r"^[ \t\n\v\f\r]*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))",
                    re.IGNORECASE)
_INT = re.compile(r"^[ \t\n\v\f\r]*([+-]?\d+)")


def _stod(s: str) -> float:
    m = _FLOAT.match(s)
    if not m:
        raise ValueError(f"stod: no conversion for {s!r}")
    return float(m.group(1))


def _stoi(s: str) -> int:
    m = _INT.match(s)
    if not m:
        raise ValueError(f"stoi: no conversion for {s!r}")
    v = int(m.group(1))
    if not -2 ** 31 <= v < 2 ** 31:
        raise ValueError(f"stoi: out of range {s!r}")
    return v


@dataclass
class ModelConfig:
    """seismic::ModelConfig (core/config.h:21-31)."""
    vp_min: float = 1450.0
    vp_max: float = 8500.0
    vs_min: float = 0.0
    vs_max: float = 5000.0
    rho_min: float = 1000.0
    rho_max: float = 3300.0
    initial_vp: float = 1500.0
    initial_vs: float = 0.0
    initial_rho: float = 2200.0


@dataclass
class InversionConfig:
    """seismic::InversionConfig (core/config.h:33-43)."""
    max_iterations: int = 50
    step_length: float = 0.01
    gradient_smoothing_sigma: float = 2.0
    regularization_lambda: float = 1e-4
    misfit_tolerance: float = 1e-6
    misfit_type: str = "cross_correlation"
    gradient_precondition: int = 1
    line_search_max: int = 10
    line_search_factor: float = 0.5


@dataclass
class TomographyConfig:
    """seismic::TomographyConfig (core/config.h:45-51)."""
    solver: SolverConfig = field(default_factory=SolverConfig)
    model: ModelConfig = field(default_factory=ModelConfig)
    inversion: InversionConfig = field(default_factory=InversionConfig)
    obs_stations: dict = field(default_factory=dict)
    source_positions: list = field(default_factory=list)


_WS = " \t\r\n"


def load_config(yaml_path: str) -> TomographyConfig:
    cfg = TomographyConfig()
    try:
        fh = open(yaml_path, "r")
    except OSError:
        return cfg
    section = ""
    with fh:
        for raw in fh.read().split("\n"):
            line = raw.lstrip(_WS).rstrip(_WS)
            if not line or line[0] == "#":
                continue
            if line[-1] == ":":
                section = line[:-1]
                continue
            pos = line.find(":")
            if pos < 0:
                continue
            key = line[:pos].strip(" \t")
            val = line[pos + 1:].strip(" \t")
            s, m, inv = cfg.solver, cfg.model, cfg.inversion
            if section == "solver":
                if key == "frequency": s.frequency = _stod(val)
                elif key == "dt": s.dt = _stod(val)
                elif key == "nt": s.nt = _stoi(val)
                elif key == "water_depth": s.water_depth = _stod(val)
                elif key == "sponge_width": s.sponge_width = _stoi(val)
                elif key == "sponge_damping": s.sponge_damping = _stod(val)
            elif section == "model":
                if key == "vp_min": m.vp_min = _stod(val)
                elif key == "vp_max": m.vp_max = _stod(val)
                elif key == "initial_vp": m.initial_vp = _stod(val)
                elif key == "initial_vs": m.initial_vs = _stod(val)
                elif key == "initial_rho": m.initial_rho = _stod(val)
            elif section == "inversion":
                if key == "max_iterations": inv.max_iterations = _stoi(val)
                elif key == "step_length": inv.step_length = _stod(val)
                elif key == "gradient_smoothing_sigma": inv.gradient_smoothing_sigma = _stod(val)
                elif key == "regularization_lambda": inv.regularization_lambda = _stod(val)
                elif key == "misfit_type": inv.misfit_type = val
    return cfg


def config_vector(c: TomographyConfig) -> list:
    """The 17 values the fixture generator records, in its order."""
    return [c.solver.frequency, c.solver.dt, c.solver.nt, c.solver.water_depth, c.solver.seafloor_gradient,
            c.solver.sponge_width, c.solver.sponge_damping, c.solver.snapshot_interval, c.model.vp_min,
            c.model.vp_max, c.model.initial_vp, c.model.initial_vs, c.model.initial_rho,
            c.inversion.max_iterations, c.inversion.step_length, c.inversion.gradient_smoothing_sigma,
            c.inversion.regularization_lambda]
