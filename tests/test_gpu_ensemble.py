"""Ensembles of uneven grids: every group's members batched into one launch per
stage, all groups' RK4 integration captured into one CUDA graph.  Each member
must step exactly as a single-state handle steps it (same kernels, same
arithmetic, bit for bit when both use the same FFT variants)."""
import numpy as np
import pytest

import wv_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available()
    build.build()
    return wvgpu


def _cfg(wv, Nx, Nz):
    # 3.125 km per grid point, Lz = 4 km (the ensemble workload's domains)
    return wv.Configuration(Nx=Nx, Ny=Nx, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Nx, Lz=4000.0,
                            latitude=33.0)


GROUPS = [(64, 33, 3), (32, 17, 2), (48, 25, 2)]


def _members(wv, precision, groups=GROUPS, seed0=100):
    """Per group: configuration, single-state kernel, stacked member states and dt."""
    import torch
    out = []
    seed = seed0
    for Nx, Nz, B in groups:
        cfg = _cfg(wv, Nx, Nz)
        k = wv.WVTransformConstantStratificationKernel(cfg, precision=precision)
        states, dts = [], []
        for m in range(B):
            urms = 0.05 + 0.15 * m / max(B - 1, 1)
            A = wv.synthetic_state(k, seed=seed, urms=urms)
            seed += 1
            dts.append(wv.cfl_time_step(k, *A))
            states.append(np.stack(A))
        X = torch.from_numpy(np.ascontiguousarray(np.stack(states))).cuda()
        out.append((cfg, k, X, min(dts)))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ensemble_members_equal_single_state_runs(wv, precision):
    import torch
    groups = _members(wv, precision)
    ens = wv.WVEnsemble([g[0] for g in groups], [g[2].shape[0] for g in groups], precision=precision, autotune=False)
    X = [g[2].clone() for g in groups]
    dts = [g[3] for g in groups]
    steps = 3
    t1 = ens.rk4(X, 0.0, 0.0, dts, steps)
    torch.cuda.synchronize()
    assert t1 == [0.0 + d + d + d for d in dts]
    for (cfg, k, X0, dt), Xe in zip(groups, X):
        for m in range(X0.shape[0]):
            s = [X0[m, c].clone() for c in range(3)]
            k.rk4(*s, 0.0, 0.0, dt, steps)
            torch.cuda.synchronize()
            for c in range(3):
                assert torch.equal(s[c], Xe[m, c]), (cfg.Nx, m, c)
        k.close()
    met = ens.metrics()
    assert met["graph_launches"] == 1 and met["graph_captures"] == 1
    assert met["member_steps"] == steps * sum(g[2].shape[0] for g in groups)
    ens.close()


def test_ensemble_autotune_and_graph_update(wv):
    import torch
    groups = _members(wv, "mixed", seed0=200)
    ens = wv.WVEnsemble([g[0] for g in groups], [g[2].shape[0] for g in groups], precision="mixed", autotune=True)
    tune = ens.tuning()
    print("ensemble autotune:", tune)
    # the 64 grid has warp and Stockham variants on both axes (4 candidates); 48
    # has Stockham only (1).  Every vertical kernel the grid has is timed per
    # direction, and the fastest of each direction kept.
    assert tune[0]["warp_y_available"] and tune[0]["warp_x_available"] and len(tune[0]["candidate_ms"]) == 4
    assert len(tune[2]["candidate_ms"]) == 1
    assert not tune[2]["warp_y_available"] and not tune[2]["warp_x_available"]
    for tn in tune:
        assert set(tn["vertical_inverse_ms"]) == {"cuda", "fft", "tensor"} and set(tn["vertical_forward_ms"]) >= {"cuda", "fft"}
        assert tn["vertical"] == min(tn["vertical_inverse_ms"], key=tn["vertical_inverse_ms"].get)
        assert tn["vertical_forward"] == min(tn["vertical_forward_ms"], key=tn["vertical_forward_ms"].get)
    X = [g[2].clone() for g in groups]
    dts = [g[3] for g in groups]
    t = ens.rk4(X, 0.0, 0.0, dts, 2)
    t = ens.rk4(X, t, 0.0, dts, 2)  # same topology, new times: graph updated in place
    torch.cuda.synchronize()
    met = ens.metrics()
    assert met["graph_captures"] == 2 and met["graph_instantiations"] == 1 and met["graph_updates"] == 1
    for (cfg, k, X0, dt), Xe, tg, tn in zip(groups, X, t, tune):
        k.set_vertical_kernels(tn["vertical"], tn["vertical_forward"])  # the group's kernels (FP32 variants differ in rounding)
        for m in range(X0.shape[0]):
            s = [X0[m, c].clone() for c in range(3)]
            tt = k.rk4(*s, 0.0, 0.0, dt, 4)[3]
            torch.cuda.synchronize()
            assert tt == tg
            for c in range(3):
                ref = s[c].cpu().numpy()
                got = Xe[m, c].cpu().numpy()
                scale = max(float(np.max(np.abs(ref))), 1e-300)
                assert float(np.max(np.abs(got - ref))) <= 1e-4 * scale, (cfg.Nx, m, c)
        k.close()
    ens.close()


def test_ensemble_rejects_bad_states(wv):
    import torch
    cfg = _cfg(wv, 32, 17)
    ens = wv.WVEnsemble([cfg, cfg], [2, 1], precision="fp64", autotune=False)
    shp = ens.state_shapes
    good = [torch.zeros(s, dtype=torch.complex128, device="cuda") for s in shp]
    with pytest.raises(wv.WVKernelError) as e:
        ens.rk4([good[0], torch.zeros(shp[0], dtype=torch.complex128, device="cuda")], 0.0, 0.0, 10.0, 1)
    assert e.value.code == 2
    # overlapping group states
    big = torch.zeros((3,) + shp[0][1:], dtype=torch.complex128, device="cuda")
    with pytest.raises(wv.WVKernelError) as e:
        ens.rk4([big[0:2], big[1:2]], 0.0, 0.0, 10.0, 1)
    assert e.value.code == 4
    with pytest.raises(wv.WVKernelError) as e:
        ens.rk4(good, 0.0, 0.0, -1.0, 1)
    assert e.value.code == 1
    ens.close()
