"""Python host binding of the GB300 constant-stratification spectral step.

Mirrors the reference's kernel interface
(CompiledKernel/include/WaveVortexKernel/WVTransformConstantStratificationKernel.hpp:47-110)
on top of the C ABI in include/wvgpu.h: same operation names, same argument
meaning, and failures raised with the reference's status codes and messages.

Coefficient arrays are complex128 of shape (Nkl, Nj) -- the same memory as
the reference's column-major [Nj, Nkl] WVComplex64 arrays; field bundles are
float64 of shape (nfield, Nz, Ny, Nx) -- the same memory as [Nx, Ny, Nz, nfield].
numpy arrays go through the host-pointer entry points; CUDA torch tensors
through the device-pointer entry points on the current torch stream.

There is no CPU fallback: if libwvgpu.so is missing or no GPU is present,
operations raise.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwvgpu.so")

CONTRACT_VERSION = 4
PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_FP32X2 = 2
FORCING_NONLINEAR_ADVECTION = 1
FORCING_ADAPTIVE_DAMPING = 2

# WVKernelStatusCode (CompiledKernel/include/WaveVortexKernel/WVKernelTypes.hpp:22-35)
STATUS_NAMES = ["success", "invalidConfiguration", "invalidShape", "invalidPointer", "overlappingArrays", "sizeOverflow",
                "allocationFailure", "fftPlanFailure", "fftExecutionFailure", "numericalFailure", "unsupportedOperation",
                "reentrantExecution"]

# MATLAB error identifiers of the gateway (wv_compiled_backend_mex.cpp:61-77)
_IDENTIFIERS = {1: "WaveVortexModel:CompiledKernelInvalidConfiguration", 2: "WaveVortexModel:CompiledKernelShape",
                3: "WaveVortexModel:CompiledKernelOwnership", 4: "WaveVortexModel:CompiledKernelOwnership",
                5: "WaveVortexModel:CompiledKernelSizeOverflow", 6: "WaveVortexModel:CompiledKernelAllocation",
                7: "WaveVortexModel:CompiledKernelPlan", 8: "WaveVortexModel:CompiledKernelExecution",
                9: "WaveVortexModel:CompiledKernelNumericalFailure", 10: "WaveVortexModel:CompiledKernelUnsupportedOperation",
                11: "WaveVortexModel:CompiledKernelReentrantExecution"}


class WVKernelError(RuntimeError):
    def __init__(self, code, message):
        self.code = int(code)
        self.status = STATUS_NAMES[self.code] if 0 <= self.code < len(STATUS_NAMES) else "unknown"
        self.identifier = _IDENTIFIERS.get(self.code, "WaveVortexModel:CompiledKernelFailure")
        super().__init__(f"{self.identifier}: {message}")


class _Config(ctypes.Structure):
    _fields_ = [("contract_version", ctypes.c_uint32), ("Nx", ctypes.c_uint64), ("Ny", ctypes.c_uint64),
                ("Nz", ctypes.c_uint64), ("Nj", ctypes.c_uint64), ("Lx", ctypes.c_double), ("Ly", ctypes.c_double),
                ("Lz", ctypes.c_double), ("N0", ctypes.c_double), ("rho0", ctypes.c_double), ("g", ctypes.c_double),
                ("planetary_radius", ctypes.c_double), ("rotation_rate", ctypes.c_double), ("latitude", ctypes.c_double),
                ("is_hydrostatic", ctypes.c_uint8), ("should_antialias", ctypes.c_uint8)]


class _Sizes(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("Nx", "Ny", "Nz", "Nj", "Nkl", "NxHalf", "M", "active_rows", "kx_columns",
                                               "device_bytes")]


class _StageTimes(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("vertical_inverse_ms", "y_inverse_ms", "x_products_ms", "y_forward_ms",
                                               "vertical_forward_ms")] + [("fluxes", ctypes.c_uint64)]


_VKIND = {0: "cuda", 1: "tensor", 2: "fft"}  # WV_VERTICAL_*
_VCODE = {v: k for k, v in _VKIND.items()}


class _EnsembleTuning(ctypes.Structure):
    _fields_ = [("warp_y_available", ctypes.c_int), ("warp_x_available", ctypes.c_int),
                ("tensor_vertical_available", ctypes.c_int), ("stockham_y", ctypes.c_int), ("stockham_x", ctypes.c_int),
                ("vertical", ctypes.c_int), ("vertical_forward", ctypes.c_int), ("candidates", ctypes.c_int),
                ("candidate_ms", ctypes.c_float * 12), ("vertical_inverse_ms", ctypes.c_float * 3),
                ("vertical_forward_ms", ctypes.c_float * 3), ("flux_ms", ctypes.c_float)]


class _EnsembleMetrics(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("graph_captures", "graph_instantiations", "graph_updates",
                                               "graph_launches", "kernel_launches", "member_steps", "device_bytes")]


class _Metrics(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("nonlinear_flux_calls", "rhs_evaluations", "forward_calls", "inverse_calls",
                                               "rk4_steps", "kernel_launches", "device_bytes")] + \
               [("last_max_horizontal_speed", ctypes.c_double)]


class _RK23Options(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("relative_tolerance", "absolute_tolerance_scale", "safety_factor",
                                               "rejection_floor_factor", "maximum_step_factor", "maximum_step_size")] + \
               [("maximum_recorded_step_diagnostics", ctypes.c_uint64)]


class _RK23Diagnostic(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("initial_time", "accepted_step_size", "normalized_error",
                                               "next_step_size")] + \
               [("rejected_attempt_count", ctypes.c_uint64), ("rhs_evaluation_count", ctypes.c_uint64),
                ("reused_fsal_derivative", ctypes.c_uint8)]


class _RK23Metrics(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("rhs_evaluations", "accepted_steps", "rejected_steps", "fsal_reuses",
                                               "fsal_invalidations", "rejected_initial_derivative_reuses",
                                               "dense_output_evaluations")] + \
               [(n, ctypes.c_double) for n in ("last_proposed_step_size", "last_accepted_step_size", "normalized_error",
                                               "next_step_size")] + [("workspace_bytes", ctypes.c_uint64)]


class _ParticleGroup(ctypes.Structure):
    _fields_ = [("count", ctypes.c_uint64), ("xy_only", ctypes.c_int), ("interpolation", ctypes.c_int),
                ("z_fixed", ctypes.c_void_p), ("horizontal_tolerance", ctypes.c_double),
                ("vertical_tolerance", ctypes.c_double)]


class _Tracer(ctypes.Structure):
    _fields_ = [("antialias", ctypes.c_int), ("absolute_tolerance", ctypes.c_double)]


@dataclass
class Configuration:
    """WVTransformConstantStratificationConfiguration (WVKernelTypes.hpp:129-146)."""

    Nx: int
    Ny: int
    Nz: int
    Nj: int
    Lx: float
    Ly: float
    Lz: float
    N0: float = 5.2e-3
    rho0: float = 1025.0
    g: float = 9.81
    planetaryRadius: float = 6.371e6
    rotationRate: float = 7.2921e-5
    latitude: float = 33.0
    isHydrostatic: bool = False
    shouldAntialias: bool = True
    contractVersion: int = CONTRACT_VERSION

    def _c(self):
        return _Config(self.contractVersion, self.Nx, self.Ny, self.Nz, self.Nj, self.Lx, self.Ly, self.Lz, self.N0,
                       self.rho0, self.g, self.planetaryRadius, self.rotationRate, self.latitude,
                       int(bool(self.isHydrostatic)), int(bool(self.shouldAntialias)))


_lib = None


def library_path():
    return LIB_PATH


def load_library():
    """Loads libwvgpu.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libwvgpu.so not found at {LIB_PATH}; build it with wvgpu.build.build()")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    D = ctypes.c_double
    lib.wv_describe.argtypes = [ctypes.POINTER(_Config), ctypes.POINTER(_Sizes), ctypes.c_char_p, ctypes.c_size_t]
    lib.wv_describe_modes.argtypes = [ctypes.POINTER(_Config), P, P, P, P, P]
    lib.wv_create.argtypes = [ctypes.POINTER(_Config), ctypes.c_int, ctypes.POINTER(P)]
    lib.wv_destroy.argtypes = [P]
    lib.wv_destroy.restype = None
    lib.wv_last_message.argtypes = [P]
    lib.wv_last_message.restype = ctypes.c_char_p
    lib.wv_get_sizes.argtypes = [P, ctypes.POINTER(_Sizes)]
    lib.wv_get_metrics.argtypes = [P, ctypes.POINTER(_Metrics)]
    lib.wv_set_forcing.argtypes = [P, ctypes.c_uint32]
    lib.wv_set_stage_instrumentation.argtypes = [P, ctypes.c_int]
    lib.wv_set_vertical_kernel.argtypes = [P, ctypes.c_int]
    lib.wv_get_vertical_kernel.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    lib.wv_set_vertical_kernels.argtypes = [P, ctypes.c_int, ctypes.c_int]
    lib.wv_set_fft_variants.argtypes = [P, ctypes.c_int, ctypes.c_int]
    lib.wv_get_fft_variants.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.wv_get_vertical_kernels.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.wv_get_device_status.argtypes = [P, ctypes.POINTER(ctypes.c_uint)]
    lib.wv_reset_device_status.argtypes = [P]
    lib.wv_error_tolerances.argtypes = [P, D, P, P]
    # test hooks (failure injection for the contract tests)
    lib.wv_test_fail_allocation_after.argtypes = [ctypes.c_longlong]
    lib.wv_test_live_device_bytes.argtypes = []
    lib.wv_test_live_device_bytes.restype = ctypes.c_longlong
    lib.wv_test_fail_launch_after.argtypes = [P, ctypes.c_longlong]
    lib.wv_test_hold_busy.argtypes = [P, ctypes.c_int]
    lib.wv_test_inject_wait_timeout.argtypes = [P, ctypes.c_uint]
    lib.wv_get_stage_times.argtypes = [P, ctypes.POINTER(_StageTimes)]
    for name in ("wv_nonlinear_flux", "wv_evaluate_rhs"):
        getattr(lib, name).argtypes = [P, D, D, P, P, P, P, P, P]
    for name in ("wv_nonlinear_flux_device", "wv_evaluate_rhs_device", "wv_nonlinear_flux_device_noalloc"):
        getattr(lib, name).argtypes = [P, D, D, P, P, P, P, P, P, P]
    lib.wv_forward.argtypes = [P, P, D, D, P, P, P]
    lib.wv_forward_device.argtypes = [P, P, D, D, P, P, P, P]
    lib.wv_inverse.argtypes = [P, D, D, P, P, P, P]
    lib.wv_inverse_device.argtypes = [P, D, D, P, P, P, P, P]
    lib.wv_inverse_uvw.argtypes = [P, D, D, P, P, P, P]
    lib.wv_field_derivatives.argtypes = [P, D, D, P, P, P, ctypes.c_int, P]
    lib.wv_field_derivatives_device.argtypes = [P, D, D, P, P, P, ctypes.c_int, P, P]
    lib.wv_advect_fgrid_scalar.argtypes = [P, P, P, ctypes.c_int, P]
    lib.wv_family_derivatives.argtypes = [P, ctypes.c_int, P, P, P]
    lib.wv_family_derivatives_device.argtypes = [P, ctypes.c_int, P, P, P, P]
    lib.wv_advect_fgrid_scalar_device.argtypes = [P, P, P, ctypes.c_int, P, P]
    lib.wv_inverse_uvw_device.argtypes = [P, D, D, P, P, P, P, P]
    for name in ("wv_nonlinear_flux_with_advection_fields", "wv_nonlinear_flux_using_advection_fields"):
        getattr(lib, name).argtypes = [P, D, D, P, P, P, P, P, P, P]
        getattr(lib, name + "_device").argtypes = [P, D, D, P, P, P, P, P, P, P, P]
    lib.wv_rk4_steps.argtypes = [P, P, P, P, ctypes.POINTER(D), D, D, ctypes.c_int]
    lib.wv_rk4_steps_device.argtypes = [P, P, P, P, ctypes.POINTER(D), D, D, ctypes.c_int, P]
    lib.wv_rk4_set_dense_output.argtypes = [P, ctypes.c_int]
    lib.wv_rk4_advance_to_time_device.argtypes = [P, P, P, P, ctypes.POINTER(D), D, D, D, P]
    lib.wv_rk4_advance_to_time.argtypes = [P, P, P, P, ctypes.POINTER(D), D, D, D]
    lib.wv_rk4_dense_output_device.argtypes = [P, D, P, P, P, P]
    lib.wv_flux_vjp_device.argtypes = [P, D, D, P, P, P, P, P, P, P, P, P, P]
    lib.wv_inverse_vjp_device.argtypes = [P, D, D, P, P, P, P, P]
    lib.wv_rk4_step_vjp_device.argtypes = [P, P, P, P, D, D, D, P, P, P, P]
    lib.wv_rk4_adjoint_device.argtypes = [P, P, P, P, D, D, D, ctypes.c_int, ctypes.c_int, P, P, P, P]
    lib.wv_ensemble_create.argtypes = [ctypes.POINTER(_Config), ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.POINTER(P)]
    lib.wv_ensemble_destroy.argtypes = [P]
    lib.wv_ensemble_destroy.restype = None
    lib.wv_ensemble_last_message.argtypes = [P]
    lib.wv_ensemble_last_message.restype = ctypes.c_char_p
    lib.wv_ensemble_get_sizes.argtypes = [P, ctypes.c_int, ctypes.POINTER(_Sizes)]
    lib.wv_ensemble_get_tuning.argtypes = [P, ctypes.c_int, ctypes.POINTER(_EnsembleTuning)]
    lib.wv_ensemble_get_metrics.argtypes = [P, ctypes.POINTER(_EnsembleMetrics)]
    lib.wv_ensemble_set_vertical_kernel.argtypes = [P, ctypes.c_int]
    lib.wv_ensemble_rk4_device.argtypes = [P, ctypes.POINTER(P), ctypes.POINTER(D), D, ctypes.POINTER(D), ctypes.c_int, P]
    lib.wv_rk23_default_options.argtypes = [ctypes.POINTER(_RK23Options)]
    lib.wv_rk23_default_options.restype = None
    lib.wv_rk23_create.argtypes = [P, ctypes.POINTER(_RK23Options), ctypes.POINTER(P)]
    lib.wv_rk23_destroy.argtypes = [P]
    lib.wv_rk23_destroy.restype = None
    lib.wv_rk23_last_message.argtypes = [P]
    lib.wv_rk23_last_message.restype = ctypes.c_char_p
    lib.wv_rk23_prepare_after_restart.argtypes = [P]
    lib.wv_rk23_step_device.argtypes = [P, P, P, P, ctypes.POINTER(D), D, D, P]
    lib.wv_rk23_advance_to_time_device.argtypes = [P, P, P, P, ctypes.POINTER(D), D, D, D, P]
    lib.wv_rk23_advance_to_time.argtypes = [P, P, P, P, ctypes.POINTER(D), D, D, D]
    lib.wv_rk23_dense_output_device.argtypes = [P, D, P, P, P, P]
    lib.wv_rk23_next_step_size.argtypes = [P, ctypes.POINTER(D)]
    lib.wv_rk23_last_accepted_step.argtypes = [P, ctypes.POINTER(D), ctypes.POINTER(D)]
    lib.wv_rk23_get_metrics.argtypes = [P, ctypes.POINTER(_RK23Metrics)]
    lib.wv_rk23_get_diagnostics.argtypes = [P, ctypes.POINTER(_RK23Diagnostic), ctypes.c_uint64,
                                            ctypes.POINTER(ctypes.c_uint64)]
    lib.wv_rk23_tolerance_hash.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    lib.wv_rk23_create_for_system.argtypes = [P, ctypes.POINTER(_RK23Options), ctypes.POINTER(P)]
    lib.wv_rk23_system_step_device.argtypes = [P, P, ctypes.POINTER(D), D, D, P]
    lib.wv_rk23_system_advance_to_time_device.argtypes = [P, P, ctypes.POINTER(D), D, D, D, P]
    lib.wv_rk23_system_dense_output_device.argtypes = [P, D, P, P]
    lib.wv_system_create.argtypes = [P, ctypes.POINTER(_ParticleGroup), ctypes.c_int, ctypes.POINTER(_Tracer), ctypes.c_int,
                                     ctypes.POINTER(P)]
    lib.wv_system_destroy.argtypes = [P]
    lib.wv_system_destroy.restype = None
    lib.wv_system_last_message.argtypes = [P]
    lib.wv_system_last_message.restype = ctypes.c_char_p
    lib.wv_system_get_layout.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64), P, P,
                                         ctypes.c_uint64]
    lib.wv_system_rhs_device.argtypes = [P, D, D, P, P, P]
    lib.wv_system_rk4_device.argtypes = [P, P, ctypes.POINTER(D), D, D, ctypes.c_int, P]
    lib.wv_system_rk4.argtypes = [P, P, ctypes.POINTER(D), D, D, ctypes.c_int]
    _lib = lib
    return lib


def exported_symbols():
    """Names of the C entry points this binding expects (declared in include/wvgpu.h)."""
    return ["wv_describe", "wv_describe_modes", "wv_create", "wv_destroy", "wv_last_message", "wv_get_sizes",
            "wv_get_metrics", "wv_set_forcing", "wv_set_stage_instrumentation", "wv_get_stage_times",
            "wv_set_vertical_kernel", "wv_get_vertical_kernel", "wv_set_vertical_kernels", "wv_get_vertical_kernels",
            "wv_set_fft_variants", "wv_get_fft_variants",
            "wv_get_device_status", "wv_reset_device_status", "wv_error_tolerances",
            "wv_test_fail_allocation_after", "wv_test_live_device_bytes", "wv_test_fail_launch_after", "wv_test_hold_busy",
            "wv_test_inject_wait_timeout", "wv_nonlinear_flux", "wv_evaluate_rhs", "wv_forward", "wv_inverse",
            "wv_rk4_steps", "wv_nonlinear_flux_device", "wv_evaluate_rhs_device", "wv_forward_device",
            "wv_inverse_device", "wv_rk4_steps_device", "wv_nonlinear_flux_device_noalloc", "wv_flux_vjp_device",
            "wv_inverse_vjp_device", "wv_rk4_step_vjp_device", "wv_rk4_adjoint_device",
            "wv_nonlinear_flux_with_advection_fields", "wv_nonlinear_flux_using_advection_fields", "wv_inverse_uvw",
            "wv_nonlinear_flux_with_advection_fields_device", "wv_nonlinear_flux_using_advection_fields_device",
            "wv_inverse_uvw_device", "wv_field_derivatives", "wv_field_derivatives_device", "wv_advect_fgrid_scalar",
            "wv_advect_fgrid_scalar_device", "wv_family_derivatives", "wv_family_derivatives_device", "wv_ensemble_create",
            "wv_ensemble_destroy", "wv_ensemble_last_message", "wv_ensemble_get_sizes", "wv_ensemble_get_tuning",
            "wv_ensemble_get_metrics", "wv_ensemble_set_vertical_kernel", "wv_ensemble_rk4_device",
            "wv_rk23_default_options", "wv_rk23_create", "wv_rk23_destroy", "wv_rk23_last_message",
            "wv_rk23_prepare_after_restart", "wv_rk23_step_device", "wv_rk23_advance_to_time_device",
            "wv_rk23_advance_to_time", "wv_rk23_dense_output_device", "wv_rk23_next_step_size",
            "wv_rk23_last_accepted_step", "wv_rk23_get_metrics", "wv_rk23_get_diagnostics", "wv_rk23_tolerance_hash",
            "wv_rk23_create_for_system", "wv_rk23_system_step_device", "wv_rk23_system_advance_to_time_device",
            "wv_rk23_system_dense_output_device", "wv_system_create", "wv_system_destroy", "wv_system_last_message",
            "wv_system_get_layout", "wv_system_rhs_device", "wv_system_rk4_device", "wv_system_rk4",
            "wv_rk4_set_dense_output", "wv_rk4_advance_to_time_device", "wv_rk4_advance_to_time",
            "wv_rk4_dense_output_device"]


def describe(configuration: Configuration):
    """Validates a configuration on the host and returns its sizes (no GPU needed)."""
    lib = load_library()
    s = _Sizes()
    buf = ctypes.create_string_buffer(512)
    rc = lib.wv_describe(ctypes.byref(configuration._c()), ctypes.byref(s), buf, 512)
    if rc != 0:
        raise WVKernelError(rc, buf.value.decode())
    return {n: int(getattr(s, n)) for n, _ in _Sizes._fields_}


def describe_modes(configuration: Configuration):
    """Canonical WV mode order and dispersion relation built on the host."""
    lib = load_library()
    s = describe(configuration)
    Nkl, M = s["Nkl"], s["M"]
    kMode = np.zeros(Nkl, np.int64)
    lMode = np.zeros(Nkl, np.int64)
    omega = np.zeros(M)
    rows = np.zeros(Nkl, np.uint64)
    conj = np.zeros(Nkl, np.uint8)
    rc = lib.wv_describe_modes(ctypes.byref(configuration._c()), kMode.ctypes.data, lMode.ctypes.data, omega.ctypes.data,
                               rows.ctypes.data, conj.ctypes.data)
    if rc != 0:
        raise WVKernelError(rc, "descriptor construction failed")
    return dict(kMode=kMode, lMode=lMode, omega=omega.reshape(Nkl, s["Nj"]), storageRow=rows.astype(np.int64),
                conjugated=conj.astype(bool))


def _is_torch(x):
    return type(x).__module__.startswith("torch")


class WVTransformConstantStratificationKernel:
    """GPU kernel handle with the reference kernel's operations."""

    def __init__(self, configuration: Configuration, precision: str = "fp64"):
        lib = load_library()
        self.configuration = configuration
        self.precision = precision
        p = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED, "fp32x2": PRECISION_FP32X2}[precision]
        h = ctypes.c_void_p()
        rc = lib.wv_create(ctypes.byref(configuration._c()), p, ctypes.byref(h))
        if rc != 0:
            msg = "GPU kernel creation failed"
            try:
                describe(configuration)
            except WVKernelError as e:
                raise e
            raise WVKernelError(rc, msg)
        self._h = h
        self._lib = lib
        s = _Sizes()
        lib.wv_get_sizes(h, ctypes.byref(s))
        self.sizes = {n: int(getattr(s, n)) for n, _ in _Sizes._fields_}
        self.Nkl = self.sizes["Nkl"]
        self.Nj = configuration.Nj
        self.spectral_shape = (self.Nkl, self.Nj)
        self.spatial_shape = (configuration.Nz, configuration.Ny, configuration.Nx)

    @classmethod
    def create(cls, configuration: Configuration, precision: str = "fp64"):
        return cls(configuration, precision)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.wv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise WVKernelError(rc, self._lib.wv_last_message(self._h).decode())

    # -- helpers --------------------------------------------------------------------
    def _host_coeff(self, a, name):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        if a.shape != self.spectral_shape:
            raise WVKernelError(2, f"{name} must have shape [Nj,Nkl].")
        return a

    def _dev_coeff(self, a, name):
        import torch
        if a.dtype != torch.complex128 or tuple(a.shape) != self.spectral_shape or not a.is_contiguous():
            raise WVKernelError(2, f"{name} must be a contiguous complex128 [Nj,Nkl] tensor.")
        return a

    @staticmethod
    def _stream():
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    # -- operations ----------------------------------------------------------------------
    def set_forcing(self, nonlinear=True, adaptive_damping=False):
        flags = (FORCING_NONLINEAR_ADVECTION if nonlinear else 0) | (FORCING_ADAPTIVE_DAMPING if adaptive_damping else 0)
        self._check(self._lib.wv_set_forcing(self._h, flags))

    def nonlinearFlux(self, t, t0, Ap, Am, A0, out=None, scheduled=False):
        """nonlinearFlux (kernel.cpp:1140-1146); with scheduled=True the forcing
        schedule's right-hand side (WVIntegrationSystem::evaluateRightHandSide)."""
        if _is_torch(Ap):
            import torch
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            F = out if out is not None else tuple(torch.empty_like(Ap) for _ in range(3))
            fn = self._lib.wv_evaluate_rhs_device if scheduled else self._lib.wv_nonlinear_flux_device
            self._check(fn(self._h, float(t), float(t0), Ap.data_ptr(), Am.data_ptr(), A0.data_ptr(), F[0].data_ptr(),
                           F[1].data_ptr(), F[2].data_ptr(), self._stream()))
            return F
        Ap, Am, A0 = (self._host_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        F = out if out is not None else tuple(np.empty(self.spectral_shape, np.complex128) for _ in range(3))
        fn = self._lib.wv_evaluate_rhs if scheduled else self._lib.wv_nonlinear_flux
        self._check(fn(self._h, float(t), float(t0), Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data, F[0].ctypes.data,
                       F[1].ctypes.data, F[2].ctypes.data))
        return F

    def nonlinearFluxWithAdvectionFields(self, t, t0, Ap, Am, A0):
        """nonlinearFluxWithAdvectionFields (kernel.cpp:1148-1158): ((Fp, Fm, F0), fields (3, Nz, Ny, Nx))."""
        if _is_torch(Ap):
            import torch
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            F = tuple(torch.empty_like(Ap) for _ in range(3))
            adv = torch.empty((3,) + self.spatial_shape, dtype=torch.float64, device=Ap.device)
            self._check(self._lib.wv_nonlinear_flux_with_advection_fields_device(
                self._h, float(t), float(t0), Ap.data_ptr(), Am.data_ptr(), A0.data_ptr(), *(f.data_ptr() for f in F),
                adv.data_ptr(), self._stream()))
            return F, adv
        Ap, Am, A0 = (self._host_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        F = tuple(np.empty(self.spectral_shape, np.complex128) for _ in range(3))
        adv = np.empty((3,) + self.spatial_shape)
        self._check(self._lib.wv_nonlinear_flux_with_advection_fields(
            self._h, float(t), float(t0), Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data, *(f.ctypes.data for f in F),
            adv.ctypes.data))
        return F, adv

    def nonlinearFluxUsingAdvectionFields(self, t, t0, Ap, Am, A0, fields):
        """nonlinearFluxUsingAdvectionFields (kernel.cpp:1160-1171): the flux advected by fields (3, Nz, Ny, Nx)."""
        if _is_torch(Ap):
            import torch
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            fields = fields.contiguous()
            if tuple(fields.shape) != (3,) + self.spatial_shape or fields.dtype != torch.float64:
                raise WVKernelError(2, "Prepared advection fields must be float64 of shape [Nx,Ny,Nz,3].")
            F = tuple(torch.empty_like(Ap) for _ in range(3))
            self._check(self._lib.wv_nonlinear_flux_using_advection_fields_device(
                self._h, float(t), float(t0), Ap.data_ptr(), Am.data_ptr(), A0.data_ptr(), *(f.data_ptr() for f in F),
                fields.data_ptr(), self._stream()))
            return F
        Ap, Am, A0 = (self._host_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        fields = np.ascontiguousarray(fields, dtype=np.float64)
        if fields.shape != (3,) + self.spatial_shape:
            raise WVKernelError(2, "Prepared advection fields must be float64 of shape [Nx,Ny,Nz,3].")
        F = tuple(np.empty(self.spectral_shape, np.complex128) for _ in range(3))
        self._check(self._lib.wv_nonlinear_flux_using_advection_fields(
            self._h, float(t), float(t0), Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data, *(f.ctypes.data for f in F),
            fields.ctypes.data))
        return F

    def transformWaveVortexToUVW(self, t, t0, Ap, Am, A0):
        """transformWaveVortexToUVW (kernel.cpp:696-717): fields (3, Nz, Ny, Nx)."""
        if _is_torch(Ap):
            import torch
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            out = torch.empty((3,) + self.spatial_shape, dtype=torch.float64, device=Ap.device)
            self._check(self._lib.wv_inverse_uvw_device(self._h, float(t), float(t0), Ap.data_ptr(), Am.data_ptr(),
                                                        A0.data_ptr(), out.data_ptr(), self._stream()))
            return out
        Ap, Am, A0 = (self._host_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        out = np.empty((3,) + self.spatial_shape)
        self._check(self._lib.wv_inverse_uvw(self._h, float(t), float(t0), Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data,
                                             out.ctypes.data))
        return out

    def transformStateFieldDerivatives(self, t, t0, Ap, Am, A0, field):
        """transformStateFieldDerivatives (kernel.cpp:719-743): (d/dx, d/dy, d/dz) of
        field 0..3 / 'u', 'v', 'w', 'eta' as (3, Nz, Ny, Nx)."""
        q = {"u": 0, "v": 1, "w": 2, "eta": 3}.get(field, field)
        if _is_torch(Ap):
            import torch
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            out = torch.empty((3,) + self.spatial_shape, dtype=torch.float64, device=Ap.device)
            self._check(self._lib.wv_field_derivatives_device(self._h, float(t), float(t0), Ap.data_ptr(), Am.data_ptr(),
                                                              A0.data_ptr(), int(q), out.data_ptr(), self._stream()))
            return out
        Ap, Am, A0 = (self._host_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        out = np.empty((3,) + self.spatial_shape)
        self._check(self._lib.wv_field_derivatives(self._h, float(t), float(t0), Ap.ctypes.data, Am.ctypes.data,
                                                   A0.ctypes.data, int(q), out.ctypes.data))
        return out

    def _family(self, ffamily, Apm, A0):
        if _is_torch(Apm):
            import torch
            Apm, A0 = self._dev_coeff(Apm, "Apm"), self._dev_coeff(A0, "A0")
            out = torch.empty((4,) + self.spatial_shape, dtype=torch.float64, device=Apm.device)
            self._check(self._lib.wv_family_derivatives_device(self._h, int(ffamily), Apm.data_ptr(), A0.data_ptr(),
                                                               out.data_ptr(), self._stream()))
            return out
        Apm, A0 = self._host_coeff(Apm, "Apm"), self._host_coeff(A0, "A0")
        out = np.empty((4,) + self.spatial_shape)
        self._check(self._lib.wv_family_derivatives(self._h, int(ffamily), Apm.ctypes.data, A0.ctypes.data, out.ctypes.data))
        return out

    def transformToSpatialDomainWithFAllDerivatives(self, Apm, A0):
        """kernel.cpp:819-840: (value, d/dx, d/dy, d/dz) of the F field family, (4, Nz, Ny, Nx)."""
        return self._family(True, Apm, A0)

    def transformToSpatialDomainWithGAllDerivatives(self, Apm, A0):
        """kernel.cpp:842-863: (value, d/dx, d/dy, d/dz) of the G field family, (4, Nz, Ny, Nx)."""
        return self._family(False, Apm, A0)

    def advectFGridScalar(self, scalar, advectionFields, shouldAntialias=True):
        """advectFGridScalar (kernel.cpp:1032-1138): -(u ds/dx + v ds/dy + w ds/dz), (Nz, Ny, Nx)."""
        if _is_torch(scalar):
            import torch
            scalar = scalar.contiguous()
            adv = advectionFields.contiguous()
            if tuple(scalar.shape) != self.spatial_shape or tuple(adv.shape) != (3,) + self.spatial_shape:
                raise WVKernelError(2, "F-grid scalar input and output must have shape [Nx,Ny,Nz].")
            out = torch.empty_like(scalar)
            self._check(self._lib.wv_advect_fgrid_scalar_device(self._h, scalar.data_ptr(), adv.data_ptr(),
                                                                int(bool(shouldAntialias)), out.data_ptr(), self._stream()))
            return out
        scalar = np.ascontiguousarray(scalar, dtype=np.float64)
        adv = np.ascontiguousarray(advectionFields, dtype=np.float64)
        if scalar.shape != self.spatial_shape or adv.shape != (3,) + self.spatial_shape:
            raise WVKernelError(2, "F-grid scalar input and output must have shape [Nx,Ny,Nz].")
        out = np.empty(self.spatial_shape)
        self._check(self._lib.wv_advect_fgrid_scalar(self._h, scalar.ctypes.data, adv.ctypes.data,
                                                     int(bool(shouldAntialias)), out.ctypes.data))
        return out

    def evaluateRightHandSide(self, t, t0, Ap, Am, A0, out=None):
        return self.nonlinearFlux(t, t0, Ap, Am, A0, out=out, scheduled=True)

    def transformWaveVortexToUVWEta(self, t, t0, Ap, Am, A0, out=None):
        """transformWaveVortexToUVWEta (kernel.cpp:686-694): fields (4, Nz, Ny, Nx)."""
        shape = (4,) + self.spatial_shape
        if _is_torch(Ap):
            import torch
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            f = out if out is not None else torch.empty(shape, dtype=torch.float64, device=Ap.device)
            self._check(self._lib.wv_inverse_device(self._h, float(t), float(t0), Ap.data_ptr(), Am.data_ptr(),
                                                    A0.data_ptr(), f.data_ptr(), self._stream()))
            return f
        Ap, Am, A0 = (self._host_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        f = out if out is not None else np.empty(shape, np.float64)
        self._check(self._lib.wv_inverse(self._h, float(t), float(t0), Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data,
                                         f.ctypes.data))
        return f

    def _forward(self, fields, t, t0, nch):
        shape = (nch,) + self.spatial_shape
        if _is_torch(fields):
            import torch
            if tuple(fields.shape) != shape or fields.dtype != torch.float64 or not fields.is_contiguous():
                raise WVKernelError(2, "Fields must have shape [Nx,Ny,Nz,Nfield].")
            A = tuple(torch.empty(self.spectral_shape, dtype=torch.complex128, device=fields.device) for _ in range(3))
            self._check(self._lib.wv_forward_device(self._h, fields.data_ptr(), float(t), float(t0), A[0].data_ptr(),
                                                    A[1].data_ptr(), A[2].data_ptr(), self._stream()))
            return A
        fields = np.ascontiguousarray(fields, dtype=np.float64)
        if fields.shape != shape:
            raise WVKernelError(2, "Fields must have shape [Nx,Ny,Nz,Nfield].")
        A = tuple(np.empty(self.spectral_shape, np.complex128) for _ in range(3))
        self._check(self._lib.wv_forward(self._h, fields.ctypes.data, float(t), float(t0), A[0].ctypes.data,
                                         A[1].ctypes.data, A[2].ctypes.data))
        return A

    def transformUVWEtaToWaveVortex(self, fields, t, t0):
        """transformUVWEtaToWaveVortex (kernel.cpp:637-684), nonhydrostatic handles."""
        if self.configuration.isHydrostatic:
            raise WVKernelError(1, "transformUVWEtaToWaveVortex requires a nonhydrostatic kernel.")
        return self._forward(fields, t, t0, 4)

    def transformUVEtaToWaveVortex(self, fields, t, t0):
        """transformUVEtaToWaveVortex (kernel.cpp:583-635), hydrostatic handles."""
        if not self.configuration.isHydrostatic:
            raise WVKernelError(1, "transformUVEtaToWaveVortex requires a hydrostatic kernel.")
        return self._forward(fields, t, t0, 3)

    def rk4(self, Ap, Am, A0, t, t0, dt, steps):
        """WVFixedStepRK4::step x steps (PortableRuntime/src/WVRungeKutta.cpp:335-462).
        numpy inputs are copied; torch CUDA inputs are advanced in place.
        Returns (Ap, Am, A0, t)."""
        tt = ctypes.c_double(float(t))
        if _is_torch(Ap):
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            self._check(self._lib.wv_rk4_steps_device(self._h, Ap.data_ptr(), Am.data_ptr(), A0.data_ptr(), ctypes.byref(tt),
                                                      float(t0), float(dt), int(steps), self._stream()))
            return Ap, Am, A0, tt.value
        Ap, Am, A0 = (self._host_coeff(a, n).copy() for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        self._check(self._lib.wv_rk4_steps(self._h, Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data, ctypes.byref(tt),
                                           float(t0), float(dt), int(steps)))
        return Ap, Am, A0, tt.value

    def setRK4DenseOutput(self, enabled=True):
        """WVFixedStepRK4Options::retainDenseOutput for the RK4 entries of this handle."""
        self._check(self._lib.wv_rk4_set_dense_output(self._h, int(bool(enabled))))

    def rk4AdvanceToTime(self, Ap, Am, A0, t, t0, finalTime, dt):
        """WVFixedStepRK4::advanceToTime: steps of min(dt, finalTime - t).  torch CUDA
        inputs advance in place (returns finalTime); numpy inputs are copied
        (returns (Ap, Am, A0, finalTime))."""
        tt = ctypes.c_double(float(t))
        if _is_torch(Ap):
            Ap, Am, A0 = (self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            self._check(self._lib.wv_rk4_advance_to_time_device(self._h, Ap.data_ptr(), Am.data_ptr(), A0.data_ptr(),
                                                                ctypes.byref(tt), float(t0), float(finalTime), float(dt),
                                                                self._stream()))
            return tt.value
        Ap, Am, A0 = (self._host_coeff(a, n).copy() for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        self._check(self._lib.wv_rk4_advance_to_time(self._h, Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data,
                                                     ctypes.byref(tt), float(t0), float(finalTime), float(dt)))
        return Ap, Am, A0, tt.value

    def rk4DenseOutput(self, time):
        """WVFixedStepRK4::evaluateDenseOutput of the last RK4 step (new CUDA tensors)."""
        import torch
        out = tuple(torch.empty(self.spectral_shape, dtype=torch.complex128, device="cuda") for _ in range(3))
        self._check(self._lib.wv_rk4_dense_output_device(self._h, float(time), *(o.data_ptr() for o in out), self._stream()))
        return out

    # -- adjoint (torch CUDA tensors) ---------------------------------------------------
    def flux_vjp(self, t, t0, Ap, Am, A0, Fpb, Fmb, F0b):
        """VJP of nonlinearFlux at (Ap, Am, A0): cotangents (Apb, Amb, A0b)."""
        import torch
        ins = [self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0, Fpb, Fmb, F0b), ("Ap", "Am", "A0", "Fpb", "Fmb", "F0b"))]
        out = tuple(torch.empty_like(ins[0]) for _ in range(3))
        self._check(self._lib.wv_flux_vjp_device(self._h, float(t), float(t0), *(x.data_ptr() for x in ins),
                                                 *(o.data_ptr() for o in out), self._stream()))
        return out

    def inverse_vjp(self, t, t0, fields_bar):
        """VJP of transformWaveVortexToUVWEta: fields cotangent (4, Nz, Ny, Nx) -> (Apb, Amb, A0b)."""
        import torch
        out = tuple(torch.empty(self.spectral_shape, dtype=torch.complex128, device=fields_bar.device) for _ in range(3))
        self._check(self._lib.wv_inverse_vjp_device(self._h, float(t), float(t0), fields_bar.contiguous().data_ptr(),
                                                    *(o.data_ptr() for o in out), self._stream()))
        return out

    def rk4_step_vjp(self, Ap, Am, A0, t, t0, dt, Apb, Amb, A0b):
        """Cotangent before one RK4 step from the cotangent after it (returns new tensors)."""
        ins = [self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0"))]
        out = [self._dev_coeff(a, n).clone() for a, n in zip((Apb, Amb, A0b), ("Apb", "Amb", "A0b"))]
        self._check(self._lib.wv_rk4_step_vjp_device(self._h, *(x.data_ptr() for x in ins), float(t), float(t0), float(dt),
                                                     *(o.data_ptr() for o in out), self._stream()))
        return tuple(out)

    def rk4_adjoint(self, Ap, Am, A0, t, t0, dt, steps, checkpoint_every, Apb, Amb, A0b):
        """Cotangent at t of the state, given the cotangent at t + steps*dt (checkpointed recomputation)."""
        ins = [self._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0"))]
        out = [self._dev_coeff(a, n).clone() for a, n in zip((Apb, Amb, A0b), ("Apb", "Amb", "A0b"))]
        self._check(self._lib.wv_rk4_adjoint_device(self._h, *(x.data_ptr() for x in ins), float(t), float(t0), float(dt),
                                                    int(steps), int(checkpoint_every), *(o.data_ptr() for o in out),
                                                    self._stream()))
        return tuple(out)

    def set_vertical_kernel(self, kind):
        """'cuda' (CUDA-core dense contractions), 'tensor' (tcgen05 GEMMs: split-BF16 for both vertical
        transforms on mixed handles, exact digit slices for the vertical inverse on FP32X2 handles) or
        'fft' (FFTs of the even / odd extension over z, 3 <= Nz <= 513; the default of FP64 and FP32X2 handles)."""
        self._check(self._lib.wv_set_vertical_kernel(self._h, _VCODE[kind]))

    def vertical_kernel(self):
        """The kernel of the flux's vertical inverse transform: 'cuda', 'tensor' or 'fft'."""
        v = ctypes.c_int(0)
        self._check(self._lib.wv_get_vertical_kernel(self._h, ctypes.byref(v)))
        return _VKIND[v.value]

    def set_vertical_kernels(self, inverse, forward):
        """Kernels of the vertical inverse and forward transforms on their own ('cuda', 'tensor', 'fft')."""
        self._check(self._lib.wv_set_vertical_kernels(self._h, _VCODE[inverse], _VCODE[forward]))

    def set_fft_variants(self, y, x):
        """xy FFT kernels per axis: 'register' (warp register lines where the length allows) or 'stockham'."""
        code = {"register": 0, "stockham": 1}
        self._check(self._lib.wv_set_fft_variants(self._h, code[y], code[x]))

    def fft_variants(self):
        """(y, x) FFT kernels the flux runs: 'register' or 'stockham'."""
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self._lib.wv_get_fft_variants(self._h, ctypes.byref(a), ctypes.byref(b)))
        name = {0: "register", 1: "stockham"}
        return name[a.value], name[b.value]

    def vertical_kernels(self):
        """(inverse, forward) kernels of the flux's vertical transforms."""
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self._lib.wv_get_vertical_kernels(self._h, ctypes.byref(a), ctypes.byref(b)))
        return _VKIND[a.value], _VKIND[b.value]

    def device_status(self):
        """Device status word (bit 0: a bounded in-kernel wait ran out)."""
        v = ctypes.c_uint(0)
        self._check(self._lib.wv_get_device_status(self._h, ctypes.byref(v)))
        return int(v.value)

    def setStageInstrumentation(self, enabled):
        """setStageInstrumentation (kernel.cpp:570-581): per-stage device times."""
        self._check(self._lib.wv_set_stage_instrumentation(self._h, int(bool(enabled))))

    def stage_times(self):
        t = _StageTimes()
        self._check(self._lib.wv_get_stage_times(self._h, ctypes.byref(t)))
        return {n: getattr(t, n) for n, _ in _StageTimes._fields_}

    def metrics(self):
        m = _Metrics()
        self._check(self._lib.wv_get_metrics(self._h, ctypes.byref(m)))
        return {n: getattr(m, n) for n, _ in _Metrics._fields_}


class WVEnsemble:
    """Groups of states on uneven grids stepped together: group g holds
    members[g] states of configurations[g], each as a [members, 3, Nkl, Nj]
    complex128 CUDA tensor (Ap, Am, A0 of each member).  rk4() runs the whole
    integration of every group as one CUDA-graph launch.  No counterpart in the
    reference (one kernel object per state there)."""

    def __init__(self, configurations, members, precision: str = "mixed", autotune: bool = True):
        lib = load_library()
        if len(configurations) != len(members) or not configurations:
            raise WVKernelError(1, "One member count per configuration is required.")
        self.configurations = list(configurations)
        self.members = [int(m) for m in members]
        self.precision = precision
        p = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED, "fp32x2": PRECISION_FP32X2}[precision]
        G = len(self.configurations)
        cfgs = (_Config * G)(*(c._c() for c in self.configurations))
        mem = (ctypes.c_int * G)(*self.members)
        h = ctypes.c_void_p()
        rc = lib.wv_ensemble_create(cfgs, mem, G, p, int(bool(autotune)), ctypes.byref(h))
        if rc != 0:
            for c in self.configurations:
                describe(c)
            raise WVKernelError(rc, "GPU ensemble creation failed")
        self._h = h
        self._lib = lib
        self.sizes = []
        for g in range(G):
            s = _Sizes()
            lib.wv_ensemble_get_sizes(h, g, ctypes.byref(s))
            self.sizes.append({n: int(getattr(s, n)) for n, _ in _Sizes._fields_})
        self.state_shapes = [(m, 3, s["Nkl"], c.Nj) for m, s, c in zip(self.members, self.sizes, self.configurations)]

    def close(self):
        if getattr(self, "_h", None):
            self._lib.wv_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise WVKernelError(rc, self._lib.wv_ensemble_last_message(self._h).decode())

    def tuning(self):
        out = []
        for g in range(len(self.members)):
            t = _EnsembleTuning()
            self._check(self._lib.wv_ensemble_get_tuning(self._h, g, ctypes.byref(t)))
            out.append({"warp_y_available": bool(t.warp_y_available), "warp_x_available": bool(t.warp_x_available),
                        "tensor_vertical_available": bool(t.tensor_vertical_available),
                        "y": "stockham" if t.stockham_y or not t.warp_y_available else "warp",
                        "x": "stockham" if t.stockham_x or not t.warp_x_available else "warp",
                        "vertical": _VKIND[t.vertical], "vertical_forward": _VKIND[t.vertical_forward],
                        "candidate_ms": list(t.candidate_ms)[:max(0, min(12, t.candidates))],
                        "vertical_inverse_ms": {_VKIND[i]: v for i, v in enumerate(t.vertical_inverse_ms) if v >= 0},
                        "vertical_forward_ms": {_VKIND[i]: v for i, v in enumerate(t.vertical_forward_ms) if v >= 0},
                        "flux_ms": t.flux_ms})
        return out

    def set_vertical_kernel(self, kind):
        """'cuda', 'tensor' or 'fft' for every group (overrides the autotuner's choice)."""
        self._check(self._lib.wv_ensemble_set_vertical_kernel(self._h, _VCODE[kind]))

    def metrics(self):
        m = _EnsembleMetrics()
        self._check(self._lib.wv_ensemble_get_metrics(self._h, ctypes.byref(m)))
        return {n: int(getattr(m, n)) for n, _ in _EnsembleMetrics._fields_}

    def rk4(self, states, t, t0, dt, steps):
        """Advances every group's states in place.  t and dt: one time and one
        step per group (or a scalar for all).  Returns the groups' times after
        `steps` steps."""
        import torch
        G = len(self.members)
        if len(states) != G:
            raise WVKernelError(2, "One state tensor per group is required.")
        for x, shape in zip(states, self.state_shapes):
            if x.dtype != torch.complex128 or tuple(x.shape) != shape or not x.is_contiguous() or not x.is_cuda:
                raise WVKernelError(2, f"Group states must be contiguous complex128 CUDA tensors of shape {shape}.")
        dts = [float(dt)] * G if np.isscalar(dt) else [float(x) for x in dt]
        ts = [float(t)] * G if np.isscalar(t) else [float(x) for x in t]
        if len(dts) != G or len(ts) != G:
            raise WVKernelError(2, "One time and one step per group are required.")
        ptrs = (ctypes.c_void_p * G)(*(x.data_ptr() for x in states))
        dd = (ctypes.c_double * G)(*dts)
        tt = (ctypes.c_double * G)(*ts)
        self._check(self._lib.wv_ensemble_rk4_device(self._h, ptrs, tt, float(t0), dd, int(steps),
                                                     WVTransformConstantStratificationKernel._stream()))
        return list(tt)


@dataclass
class WVAdaptiveRK23Options:
    """WVAdaptiveRK23Options (PortableRuntime/include/WaveVortexRuntime/WVRungeKutta.hpp:112-120)."""

    relativeTolerance: float = 1e-3
    absoluteToleranceScale: float = 1e-6
    safetyFactor: float = 0.8
    rejectionFloorFactor: float = 0.5
    maximumStepFactor: float = 5.0
    maximumStepSize: float = math.inf
    maximumRecordedStepDiagnostics: int = 512

    def _c(self):
        return _RK23Options(self.relativeTolerance, self.absoluteToleranceScale, self.safetyFactor,
                            self.rejectionFloorFactor, self.maximumStepFactor, self.maximumStepSize,
                            int(self.maximumRecordedStepDiagnostics))


class WVAdaptiveRK23:
    """Adaptive Bogacki-Shampine RK23 over a kernel handle's scheduled
    right-hand side (WVAdaptiveRK23, PortableRuntime/src/WVRungeKutta.cpp:554-983):
    step(), advanceToTime(), evaluateDenseOutput(), nextStepSize(), metrics()
    and stepDiagnostics() with the reference's meaning.  States are torch CUDA
    complex128 tensors advanced in place, or numpy arrays (advanceToTime only,
    copied).  The kernel must outlive the integrator."""

    controllerIdentifier = "matlab-ode23-v1"

    def __init__(self, kernel, options: WVAdaptiveRK23Options | None = None):
        """kernel: a WVTransformConstantStratificationKernel (coefficient state) or a
        WVConstantStratificationIntegrationSystem (packed state with particles and
        tracers; step / advanceToTime / evaluateDenseOutput then take and return
        the packed CUDA state)."""
        self.system = kernel if isinstance(kernel, WVConstantStratificationIntegrationSystem) else None
        self.kernel = self.system.kernel if self.system else kernel
        self.options = options or WVAdaptiveRK23Options()
        self._lib = self.kernel._lib
        h = ctypes.c_void_p()
        if self.system:
            rc = self._lib.wv_rk23_create_for_system(self.system._h, ctypes.byref(self.options._c()), ctypes.byref(h))
        else:
            rc = self._lib.wv_rk23_create(self.kernel._h, ctypes.byref(self.options._c()), ctypes.byref(h))
        if rc != 0:
            raise WVKernelError(rc, "Adaptive RK23 creation failed (options, tolerances or device allocation).")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.wv_rk23_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise WVKernelError(rc, self._lib.wv_rk23_last_message(self._h).decode())

    def prepareStateAfterRestart(self):
        self._check(self._lib.wv_rk23_prepare_after_restart(self._h))

    def step(self, *args):
        """step(Ap, Am, A0, t, t0, proposedStepSize), or step(state, t, t0,
        proposedStepSize) for a system: one accepted step of the CUDA state (in
        place); returns the new time."""
        if self.system:
            state, t, t0, h = args
            self.system._check_state(state)
            tt = ctypes.c_double(float(t))
            self._check(self._lib.wv_rk23_system_step_device(self._h, state.data_ptr(), ctypes.byref(tt), float(t0),
                                                             float(h), self.kernel._stream()))
            return tt.value
        return self._step(*args)

    def _step(self, Ap, Am, A0, t, t0, proposedStepSize):
        Ap, Am, A0 = (self.kernel._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        tt = ctypes.c_double(float(t))
        self._check(self._lib.wv_rk23_step_device(self._h, Ap.data_ptr(), Am.data_ptr(), A0.data_ptr(), ctypes.byref(tt),
                                                  float(t0), float(proposedStepSize), self.kernel._stream()))
        return tt.value

    def advanceToTime(self, *args):
        """advanceToTime(Ap, Am, A0, t, t0, finalTime, initialStepSize): torch CUDA
        states in place (returns finalTime); numpy states are copied (returns (Ap,
        Am, A0, finalTime)).  For a system: advanceToTime(state, t, t0, finalTime,
        initialStepSize) on the packed CUDA state."""
        if self.system:
            state, t, t0, final, h = args
            self.system._check_state(state)
            tt = ctypes.c_double(float(t))
            self._check(self._lib.wv_rk23_system_advance_to_time_device(
                self._h, state.data_ptr(), ctypes.byref(tt), float(t0), float(final), float(h), self.kernel._stream()))
            return tt.value
        return self._advance(*args)

    def _advance(self, Ap, Am, A0, t, t0, finalTime, initialStepSize):
        tt = ctypes.c_double(float(t))
        if _is_torch(Ap):
            Ap, Am, A0 = (self.kernel._dev_coeff(a, n) for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
            self._check(self._lib.wv_rk23_advance_to_time_device(
                self._h, Ap.data_ptr(), Am.data_ptr(), A0.data_ptr(), ctypes.byref(tt), float(t0), float(finalTime),
                float(initialStepSize), self.kernel._stream()))
            return tt.value
        Ap, Am, A0 = (self.kernel._host_coeff(a, n).copy() for a, n in zip((Ap, Am, A0), ("Ap", "Am", "A0")))
        self._check(self._lib.wv_rk23_advance_to_time(self._h, Ap.ctypes.data, Am.ctypes.data, A0.ctypes.data,
                                                      ctypes.byref(tt), float(t0), float(finalTime),
                                                      float(initialStepSize)))
        return Ap, Am, A0, tt.value

    def evaluateDenseOutput(self, time):
        """State at `time` inside the last accepted step (new CUDA tensors; the
        packed state for a system)."""
        import torch
        if self.system:
            out = torch.empty(self.system.state_doubles, dtype=torch.float64, device="cuda")
            self._check(self._lib.wv_rk23_system_dense_output_device(self._h, float(time), out.data_ptr(),
                                                                     self.kernel._stream()))
            return out
        out = tuple(torch.empty(self.kernel.spectral_shape, dtype=torch.complex128, device="cuda") for _ in range(3))
        self._check(self._lib.wv_rk23_dense_output_device(self._h, float(time), *(o.data_ptr() for o in out),
                                                          self.kernel._stream()))
        return out

    def nextStepSize(self):
        v = ctypes.c_double()
        self._check(self._lib.wv_rk23_next_step_size(self._h, ctypes.byref(v)))
        return v.value

    def lastAcceptedStep(self):
        """(initialTime, finalTime) of the last accepted step, or None."""
        a, b = ctypes.c_double(), ctypes.c_double()
        rc = self._lib.wv_rk23_last_accepted_step(self._h, ctypes.byref(a), ctypes.byref(b))
        return None if rc == 10 else (self._check(rc), (a.value, b.value))[1]

    def metrics(self):
        m = _RK23Metrics()
        self._check(self._lib.wv_rk23_get_metrics(self._h, ctypes.byref(m)))
        return {n: getattr(m, n) for n, _ in _RK23Metrics._fields_}

    def stepDiagnostics(self):
        """List of dicts (initialTime, acceptedStepSize, normalizedError, nextStepSize,
        rejectedAttemptCount, rightHandSideEvaluationCount, reusedFSALDerivative)."""
        n = ctypes.c_uint64()
        self._check(self._lib.wv_rk23_get_diagnostics(self._h, None, 0, ctypes.byref(n)))
        buf = (_RK23Diagnostic * max(1, n.value))()
        self._check(self._lib.wv_rk23_get_diagnostics(self._h, buf, n.value, ctypes.byref(n)))
        return [dict(initialTime=d.initial_time, acceptedStepSize=d.accepted_step_size, normalizedError=d.normalized_error,
                     nextStepSize=d.next_step_size, rejectedAttemptCount=d.rejected_attempt_count,
                     rightHandSideEvaluationCount=d.rhs_evaluation_count,
                     reusedFSALDerivative=bool(d.reused_fsal_derivative)) for d in buf[:n.value]]

    def toleranceHash(self):
        """(toleranceHash, [hash of A+, A-, A0 tolerances])."""
        h = ctypes.c_uint64()
        comp = (ctypes.c_uint64 * 3)()
        self._check(self._lib.wv_rk23_tolerance_hash(self._h, ctypes.byref(h), comp))
        return h.value, list(comp)


@dataclass
class WVParticleGroup:
    """WVLagrangianParticles (PortableRuntime/include/WaveVortexRuntime/WVLagrangianParticles.hpp):
    initial positions x, y, z (z is the fixed depth of an xy-only group), the
    interpolation of the advecting velocity ("linear" or "spline") and the
    absolute tolerances of the position blocks."""

    x: object
    y: object
    z: object
    isXYOnly: bool = False
    advectionInterpolation: str = "linear"
    horizontalAbsoluteTolerance: float = 1e-5
    verticalAbsoluteTolerance: float = 1e-6


@dataclass
class WVTracerSpec:
    """A three-dimensional WVTracer (WVTracer.hpp)."""

    shouldAntialias: bool = True
    absoluteTolerance: float = 1e-8


class WVConstantStratificationIntegrationSystem:
    """Integration system with integrated observers on the GPU
    (WVConstantStratificationIntegrationSystem,
    PortableRuntime/src/WVConstantStratificationIntegrationSystem.cpp:112-400).
    The packed state (float64 CUDA tensor of `state_doubles`) holds Ap, Am, A0
    as interleaved complex, then for each particle group x, y[, z], then each
    tracer's (Nz, Ny, Nx) field.  The kernel's forcing schedule applies and the
    kernel must outlive the system."""

    def __init__(self, kernel, particles=(), tracers=()):
        self.kernel = kernel
        self._lib = kernel._lib
        self.particles = list(particles)
        self.tracers = list(tracers)
        self._z = [np.ascontiguousarray(np.asarray(g.z, dtype=np.float64)) for g in self.particles]
        groups = (_ParticleGroup * max(1, len(self.particles)))()
        for i, g in enumerate(self.particles):
            interp = {"linear": 0, "spline": 1}[g.advectionInterpolation]
            groups[i] = _ParticleGroup(len(np.asarray(g.x)), int(bool(g.isXYOnly)), interp,
                                       self._z[i].ctypes.data if g.isXYOnly else None, float(g.horizontalAbsoluteTolerance),
                                       float(g.verticalAbsoluteTolerance))
        trs = (_Tracer * max(1, len(self.tracers)))()
        for i, t in enumerate(self.tracers):
            trs[i] = _Tracer(int(bool(t.shouldAntialias)), float(t.absoluteTolerance))
        h = ctypes.c_void_p()
        rc = self._lib.wv_system_create(kernel._h, groups, len(self.particles), trs, len(self.tracers), ctypes.byref(h))
        if rc != 0:
            raise WVKernelError(rc, "Integration system creation failed.")
        self._h = h
        n = ctypes.c_uint64()
        nb = ctypes.c_uint64()
        self._lib.wv_system_get_layout(h, ctypes.byref(n), ctypes.byref(nb), None, None, 0)
        offs = np.zeros(max(1, nb.value), np.uint64)
        lens = np.zeros(max(1, nb.value), np.uint64)
        self._lib.wv_system_get_layout(h, None, None, offs.ctypes.data, lens.ctypes.data, nb.value)
        self.state_doubles = int(n.value)
        self.block_offsets = [int(v) for v in offs[:nb.value]]
        self.block_lengths = [int(v) for v in lens[:nb.value]]

    def close(self):
        if getattr(self, "_h", None):
            self._lib.wv_system_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise WVKernelError(rc, self._lib.wv_system_last_message(self._h).decode())

    def _check_state(self, state):
        import torch
        if state.dtype != torch.float64 or state.numel() != self.state_doubles or not state.is_contiguous() or not state.is_cuda:
            raise WVKernelError(2, f"The packed state must be a contiguous float64 CUDA tensor of {self.state_doubles} values.")

    def packState(self, Ap, Am, A0, tracerFields=()):
        """Packed numpy state from coefficients, the groups' initial positions and
        the tracers' initial fields (Nz, Ny, Nx)."""
        parts = [np.ascontiguousarray(a, dtype=np.complex128).view(np.float64).ravel() for a in (Ap, Am, A0)]
        for g in self.particles:
            parts += [np.asarray(g.x, np.float64), np.asarray(g.y, np.float64)]
            if not g.isXYOnly:
                parts.append(np.asarray(g.z, np.float64))
        parts += [np.asarray(f, np.float64).ravel() for f in tracerFields]
        out = np.concatenate(parts)
        if out.size != self.state_doubles:
            raise WVKernelError(2, "Packed state does not match the system layout.")
        return out

    def unpackState(self, state):
        """(Ap, Am, A0, [blocks]) views of a packed numpy state."""
        state = np.asarray(state)
        M2 = 2 * int(np.prod(self.kernel.spectral_shape))
        coeff = [state[i * M2:(i + 1) * M2].view(np.complex128).reshape(self.kernel.spectral_shape) for i in range(3)]
        return coeff[0], coeff[1], coeff[2], [state[o:o + n] for o, n in zip(self.block_offsets, self.block_lengths)]

    def evaluateRightHandSide(self, t, t0, state):
        """Right-hand side of the packed CUDA state (new tensor)."""
        import torch
        self._check_state(state)
        out = torch.empty_like(state)
        self._check(self._lib.wv_system_rhs_device(self._h, float(t), float(t0), state.data_ptr(), out.data_ptr(),
                                                   self.kernel._stream()))
        return out

    def rk4(self, state, t, t0, dt, steps):
        """WVFixedStepRK4 over the packed state: CUDA tensors in place (returns t),
        numpy arrays copied (returns (state, t))."""
        tt = ctypes.c_double(float(t))
        if _is_torch(state):
            self._check_state(state)
            self._check(self._lib.wv_system_rk4_device(self._h, state.data_ptr(), ctypes.byref(tt), float(t0), float(dt),
                                                       int(steps), self.kernel._stream()))
            return tt.value
        state = np.ascontiguousarray(state, dtype=np.float64).copy()
        if state.size != self.state_doubles:
            raise WVKernelError(2, "Packed state does not match the system layout.")
        self._check(self._lib.wv_system_rk4(self._h, state.ctypes.data, ctypes.byref(tt), float(t0), float(dt), int(steps)))
        return state, tt.value


# ---------------------------------------------------------------------------
# Synthetic states and time step through the GPU transforms (no CPU oracle).

PI = 3.141592653589793238462643383279502884


def spectral_wavenumbers(kernel):
    """Kh [Nkl] and m [Nj] of a kernel's canonical mode order."""
    c = kernel.configuration
    modes = describe_modes(c)
    k = 2.0 * PI * (modes["kMode"].astype(np.float64) / c.Lx)
    l = 2.0 * PI * (modes["lMode"].astype(np.float64) / c.Ly)
    return np.sqrt(k * k + l * l), np.arange(c.Nj) * PI / c.Lz, modes


def synthetic_state(kernel, seed, urms=0.1, t0=0.0):
    """Seeded state: uniform random phases, Gaussian amplitudes shaped by the
    isotropic spectrum (Kh^2 + m^2)^(-3/4) in amplitude (energy ~ (Kh^2+m^2)^-1.5),
    made representable by one inverse -> forward round trip on the GPU and
    scaled to the requested rms velocity (u, v, w)."""
    c = kernel.configuration
    Kh, m, _ = spectral_wavenumbers(kernel)
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = kernel.spectral_shape
    K2 = Kh[:, None] ** 2 + m[None, :] ** 2
    with np.errstate(divide="ignore"):
        env = np.where(K2 > 0, K2 ** (-0.75), 0.0)
    comps = []
    for _ in range(3):
        amp = rng.standard_normal(shape) * env
        ph = rng.uniform(0.0, 2.0 * PI, shape)
        comps.append(amp * np.exp(1j * ph))
    f = kernel.transformWaveVortexToUVWEta(t0, t0, *comps)
    fwd = f[[0, 1, 3]] if c.isHydrostatic else f
    A = kernel.transformUVEtaToWaveVortex(fwd, t0, t0) if c.isHydrostatic else kernel.transformUVWEtaToWaveVortex(fwd, t0, t0)
    f = kernel.transformWaveVortexToUVWEta(t0, t0, *A)
    rms = math.sqrt(float(np.mean(f[0] ** 2 + f[1] ** 2 + f[2] ** 2)))
    s = urms / rms if rms > 0 else 1.0
    return tuple(a * s for a in A)


def cfl_time_step(kernel, Ap, Am, A0, t0=0.0, cfl=0.5):
    """WVModelFixedTimeStepMethods.timeStepForCFL
    (Integrators/WVModelFixedTimeStepMethods.m:50-95): cfl times the minimum of
    dx_eff/max|u_h|, (3/2)dz/max|w| above the bottom and the fastest wave period."""
    c = kernel.configuration
    Kh, m, modes = spectral_wavenumbers(kernel)
    f = kernel.transformWaveVortexToUVWEta(t0, t0, Ap, Am, A0)
    U = float(np.max(np.sqrt(f[0] ** 2 + f[1] ** 2)))
    kk = np.abs(2.0 * PI * (modes["kMode"] / c.Lx))
    ll = np.abs(2.0 * PI * (modes["lMode"] / c.Ly))
    dx = PI / float(np.max(np.maximum(kk, ll)))
    dz = c.Lz / (c.Nz - 1)
    Wm = float(np.max(np.abs(f[2][1:])))
    advective = cfl * dx / U if U > 0 else float("inf")
    if Wm > 0:
        advective = min(advective, cfl * (1.5 * dz) / Wm)
    omax = float(np.max(np.abs(modes["omega"][:, 1:]))) if c.Nj > 1 else 0.0
    oscillatory = cfl * 2.0 * PI / omax if omax > 0 else float("inf")
    return min(advective, oscillatory)
