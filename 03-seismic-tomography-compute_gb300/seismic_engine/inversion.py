"""GPU-resident traveltime inversion driver: a drop-in for the reference's
seismic_tomography.inversion.AdjointStateInversion and FaultRecoveryPolicy
(inversion.py:22-453) with the velocity model, picks, traveltimes and
gradients kept on the device.

Per iteration, as the reference's run() (inversion.py:118-274): health check
of the model, forward model (sampled rays, bit-exact kernels), misfit,
weighted residuals, convergence test, gradient (sampled rays), NaN repair,
Gaussian smoothing (SparseOps.smooth_gradient on the device), Laplacian
regularisation (gradient.py:101-124), max-abs normalisation (:126-138),
backtracking line search (inversion.py:436-453, each trial one forward
model), update with the fault policy's clamp. The model object's vp is
updated after every iteration (the callback sees it, as in the reference);
an HDF5 writer, when given, receives the same calls with host copies.

The misfit sums and the smoothing add in a different order than numpy and
the reference's triple loop, so misfits agree to rounding (about 1e-15
relative), not bit for bit; every comparison the driver makes is the
reference's.
"""
from __future__ import annotations

import logging
import math
import time
from typing import Callable, Dict, Optional

import numpy as np

from ._lib import call
from .rays import SampledRays

logger = logging.getLogger(__name__)


class FaultRecoveryPolicy:
    """inversion.py:22-81, unchanged semantics."""

    def __init__(self, max_consecutive_faults: int = 5, nan_ratio_threshold: float = 0.1,
                 step_reduction_factor: float = 0.5, min_step_length: float = 1e-8,
                 velocity_clamp_range: tuple = (1450.0, 8500.0)):
        self.max_consecutive_faults = max_consecutive_faults
        self.nan_ratio_threshold = nan_ratio_threshold
        self.step_reduction_factor = step_reduction_factor
        self.min_step_length = min_step_length
        self.velocity_clamp_range = velocity_clamp_range
        self._consecutive_faults = 0
        self._total_faults = 0
        self._recovered_iterations = 0
        self._skipped_iterations = 0

    def should_continue(self, nan_ratio: float) -> bool:
        if self._consecutive_faults >= self.max_consecutive_faults:
            return False
        return not nan_ratio > self.nan_ratio_threshold

    def record_fault(self):
        self._consecutive_faults += 1
        self._total_faults += 1

    def record_recovery(self):
        self._recovered_iterations += 1
        self._consecutive_faults = 0

    def record_skip(self):
        self._skipped_iterations += 1

    def reduced_step_length(self, current_step: float) -> float:
        return max(current_step * self.step_reduction_factor, self.min_step_length)

    def clamp_velocity(self, vp):
        """NaN/Inf -> the lower bound, then clipped (torch or numpy)."""
        lo, hi = self.velocity_clamp_range
        if hasattr(vp, "clamp"):
            import torch
            vp = torch.where(torch.isfinite(vp), vp, torch.full_like(vp, lo))
            return vp.clamp(lo, hi)
        vp = np.where(np.isfinite(vp), vp, lo)
        return np.clip(vp, lo, hi)

    @property
    def stats(self) -> Dict:
        return {'total_faults': self._total_faults, 'consecutive_faults': self._consecutive_faults,
                'recovered_iterations': self._recovered_iterations,
                'skipped_iterations': self._skipped_iterations}


class AdjointStateInversion:
    """The reference's driver (inversion.py:84-453) over device-resident state.
    model / obs_data are the reference's VelocityModel / OBSDataCoordinator
    (read by attribute); hdf5_writer may be None. A prepared pick set may be
    passed instead of walking obs_data's picks: rays (a SampledRays built for
    the model) with the observed traveltimes and pick weights as arrays."""

    def __init__(self, model, obs_data, hdf5_writer=None, dt: float = 0.001, max_iterations: int = 50,
                 step_length: float = 0.01, smoothing_sigma: float = 2.0, regularization_lambda: float = 1e-4,
                 misfit_tolerance: float = 1e-6, misfit_type: str = "cross_correlation", line_search_max: int = 10,
                 line_search_factor: float = 0.5, enable_fault_tolerance: bool = True, device: int = 0,
                 rays: SampledRays | None = None, observed=None, weights=None):
        import torch
        self.model = model
        self.obs_data = obs_data
        self.hdf5_writer = hdf5_writer
        self.dt = dt
        self.max_iterations = max_iterations
        self.step_length = step_length
        self.smoothing_sigma = smoothing_sigma
        self.regularization_lambda = regularization_lambda
        self.misfit_tolerance = misfit_tolerance
        self.misfit_type = misfit_type
        self.line_search_max = line_search_max
        self.line_search_factor = line_search_factor
        self.enable_fault_tolerance = enable_fault_tolerance
        self.fault_policy = FaultRecoveryPolicy()
        self.device = torch.device("cuda", device)
        self.rays = rays if rays is not None else SampledRays.from_reference_objects(model, obs_data, device)
        if observed is None:
            observed = [p.travel_time for p in obs_data.picks]
        if weights is None:
            weights = [p.weight for p in obs_data.picks]
        self.observed = torch.as_tensor(np.asarray(observed, np.float64), device=self.device)
        self.weights = torch.as_tensor(np.asarray(weights, np.float64), device=self.device)
        self.shape = (model.nx, model.ny, model.nz)
        n = model.nx * model.ny * model.nz
        self._tmp = torch.empty(n, dtype=torch.float64, device=self.device)
        self._current_iteration = 0
        self._current_misfit = float('inf')
        self._misfit_history: list = []
        self._converged = False
        self._fault_events: list = []

    # ---- device helpers
    def _vp_device(self):
        import torch
        return torch.from_numpy(np.ascontiguousarray(self.model.vp, np.float64).reshape(-1)).to(self.device)

    def _set_model(self, vp):
        """VelocityModel.update_from_flat (model.py:93-95): reshape, then
        clamp_values: non-finite -> vp_min, clipped to [vp_min, vp_max]."""
        import torch
        lo, hi = self.model.vp_min, self.model.vp_max
        vp = torch.where(torch.isfinite(vp), vp, torch.full_like(vp, lo)).clamp(lo, hi)
        self.model.vp = vp.cpu().numpy().reshape(self.shape)
        return vp

    def _forward(self, vp):
        return self.rays.forward_model(vp)

    def _misfit(self, times) -> float:
        """OBSDataCoordinator.compute_misfit (obs_data.py:116-129)."""
        r = self.observed - times
        if self.misfit_type in ("l2", "cross_correlation"):
            return float(0.5 * (self.weights * (r * r)).sum())
        if self.misfit_type == "l1":
            return float((self.weights * r.abs()).sum())
        raise ValueError(f"Unknown misfit type: {self.misfit_type}")

    def _smooth(self, g):
        """SparseOps.smooth_gradient on the device (FP64)."""
        import torch
        out = torch.empty_like(g)
        nx, ny, nz = self.shape
        call("st_smooth_gradient_device", g.data_ptr(), nx, ny, nz, float(self.smoothing_sigma), out.data_ptr(),
             self._tmp.data_ptr(), torch.cuda.current_stream(self.device).cuda_stream)
        return out

    def _regularize(self, vp, g):
        """GradientComputer.apply_regularization (gradient.py:101-124)."""
        import torch
        v = vp.view(self.shape)
        lap = torch.zeros_like(v)
        lap[1:-1, :, :] += v[2:, :, :] - 2 * v[1:-1, :, :] + v[:-2, :, :]
        lap[:, 1:-1, :] += v[:, 2:, :] - 2 * v[:, 1:-1, :] + v[:, :-2, :]
        lap[:, :, 1:-1] += v[:, :, 2:] - 2 * v[:, :, 1:-1] + v[:, :, :-2]
        return g - self.regularization_lambda * lap.reshape(-1)

    @staticmethod
    def _normalize(g):
        """GradientComputer.normalize_gradient (gradient.py:126-138)."""
        m = float(g.abs().max())
        return g / m if m > 1e-30 else g

    def _write(self, name, *args):
        if self.hdf5_writer is not None:
            getattr(self.hdf5_writer, name)(*args)

    # ---- the driver
    def _verify_model_health(self, vp):
        """inversion.py:276-296."""
        import torch
        bad = int((~torch.isfinite(vp)).sum()) + int((vp < 0).sum())
        if bad > 0:
            vp = self._set_model(torch.where(torch.isfinite(vp) & (vp > 0), vp, torch.full_like(vp, 1500.0)))
        v_max = float(vp.max())
        cfl = v_max * self.dt / min(self.model.dx, self.model.dy, self.model.dz)
        if cfl > 0.5:
            logger.warning(f"CFL condition may be violated: CFL={cfl:.4f} > 0.5.")
        return vp

    def _line_search(self, vp, gradient, current_misfit: float) -> float:
        """inversion.py:436-453."""
        step = self.step_length
        for _ in range(self.line_search_max):
            trial = vp - step * gradient
            if self.enable_fault_tolerance:
                trial = self.fault_policy.clamp_velocity(trial)
            lo, hi = self.model.vp_min, self.model.vp_max  # update_from_flat's clamp, model left unchanged
            import torch
            trial = torch.where(torch.isfinite(trial), trial, torch.full_like(trial, lo)).clamp(lo, hi)
            trial_misfit = self._misfit(self._forward(trial))
            if not math.isfinite(trial_misfit):
                step *= self.fault_policy.step_reduction_factor
                continue
            if trial_misfit < current_misfit:
                return step
            step *= self.line_search_factor
        return step

    def run(self, callback: Optional[Callable] = None) -> Dict:
        import torch
        vp = self._vp_device()
        if self.enable_fault_tolerance:
            vp = self._verify_model_health(vp)
        m = self.model
        self._write("write_config", {'nx': m.nx, 'ny': m.ny, 'nz': m.nz, 'dx': m.dx, 'dy': m.dy, 'dz': m.dz,
                                     'dt': self.dt, 'max_iterations': self.max_iterations,
                                     'step_length': self.step_length, 'misfit_type': self.misfit_type,
                                     'fault_tolerance': self.enable_fault_tolerance})
        src_pos = self.obs_data.get_source_positions() if hasattr(self.obs_data, "get_source_positions") else []
        rcv_pos = self.obs_data.get_receiver_positions() if hasattr(self.obs_data, "get_receiver_positions") else []
        if len(src_pos) > 0 and len(rcv_pos) > 0:
            self._write("write_source_receiver_config", src_pos, rcv_pos)
        self._current_misfit = float('inf')
        for iteration in range(self.max_iterations):
            self._current_iteration = iteration
            t_start = time.time()
            if self.enable_fault_tolerance:
                nan_count = int((~torch.isfinite(vp)).sum())
                if nan_count > 0:
                    if not self.fault_policy.should_continue(nan_count / vp.numel()):
                        break
                    self.fault_policy.record_fault()
                    from .fields import repair_field_nan
                    host = vp.cpu().numpy().copy()
                    repair_field_nan(host, m.nx, m.ny, m.nz, halo_width=1, replace_value=1500.0)
                    vp = self._set_model(torch.from_numpy(host).to(self.device))
            times = self._forward(vp)
            misfit = self._misfit(times)
            if not math.isfinite(misfit):
                self.fault_policy.record_fault()
                self.step_length = self.fault_policy.reduced_step_length(self.step_length)
                vp = self._set_model(self.fault_policy.clamp_velocity(vp))
                self._fault_events.append({'iteration': iteration, 'type': "non_finite_misfit",
                                           'detail': str(misfit), 'timestamp': time.time()})
                self.fault_policy.record_skip()
                continue
            residuals = (self.observed - times) * self.weights
            self._misfit_history.append(misfit)
            self._write("record_misfit", iteration, misfit)
            if iteration > 0:
                prev = self._misfit_history[-2]
                if abs(prev - misfit) / max(abs(prev), 1e-30) < self.misfit_tolerance:
                    self._converged = True
                    break
            gradient = self.rays.compute_gradient(vp, residuals)
            if self.enable_fault_tolerance:
                bad = int((~torch.isfinite(gradient)).sum())
                if bad > 0:
                    gradient = torch.where(torch.isfinite(gradient), gradient, torch.zeros_like(gradient))
                    self.fault_policy.record_fault()
                    self._fault_events.append({'iteration': iteration, 'type': "gradient_nan", 'detail': str(bad),
                                               'timestamp': time.time()})
            gradient = self._normalize(self._regularize(vp, self._smooth(gradient)))
            step = self._line_search(vp, gradient, misfit)
            update = vp - step * gradient
            if self.enable_fault_tolerance:
                update = self.fault_policy.clamp_velocity(update)
            vp = self._set_model(update)
            if self.enable_fault_tolerance:
                self.fault_policy.record_recovery()
            if self.hdf5_writer is not None:
                self._write("write_velocity_model", m.vp, m.nx, m.ny, m.nz, m.dx, m.dy, m.dz, iteration)
                self._write("write_gradient", gradient.cpu().numpy(), m.nx, m.ny, m.nz, iteration)
            logger.info(f"  Step length: {step:.6f}, Time: {time.time() - t_start:.2f}s")
            if callback is not None:
                callback(iteration, misfit, gradient, step)
        self._write("write_inversion_history")
        return {
            'converged': self._converged,
            'iterations': self._current_iteration + 1,
            'final_misfit': self._misfit_history[-1] if self._misfit_history else float('inf'),
            'misfit_history': self._misfit_history,
            'fault_events': self._fault_events,
            'fault_stats': self.fault_policy.stats if self.enable_fault_tolerance else None,
        }
