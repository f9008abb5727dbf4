"""The scratch-free thermal entry point (pdgpu_mctherm_static) against the workspace entry
point (pdgpu_mctherm), both called through the C ABI.

pdgpu_mctherm_static serves callers that cannot allocate device memory (their GPU memory
belongs to another runtime or pool); it keeps its workspace in a static device array inside
the library.  Both entry points run the same algorithm on the same random streams, so their
temperatures and counters must be identical, on every call: the static array keeps the last
call's contents, and each run must clear what it accumulates, whatever ran before it.  This file is collected last
so that a failure here cannot hide another test's result.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from pdspy_gb300 import _lib, thermal, workloads

pytestmark = pytest.mark.gpu


def _descriptors(models, nphot, keep, late_after=200, seed=5):
    def arr(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(C.c_double))

    descs = (_lib.ModelDesc * len(models))()
    for i, m in enumerate(models):
        r, t, p = thermal.grid_arrays(m.grid)
        sr, st = thermal._stars(m.grid)
        descs[i] = _lib.ModelDesc(len(r) - 1, len(t) - 1, len(p) - 1, arr(r), arr(t), arr(p),
                                  len(sr), arr(sr), arr(st), int(nphot))
    g = models[0].grid
    ka, ks, gg = [], [], []
    for d in g.dust:
        a, s, gv = thermal.opacity_on_grid(d, g.lam)
        ka.append(a); ks.append(s); gg.append(np.zeros_like(a) if gv is None else gv)
    dust = _lib.DustDesc(len(g.lam), len(g.dust), arr(g.lam), arr(np.stack(ka)),
                         arr(np.stack(ks)), arr(np.stack(gg)))
    opts = _lib.McOptions(seed=seed, nepoch=8, npilot=2, mrw=1, mrw_gamma=2.0, mrw_tauthres=10.0,
                          mrw_count_trigger=20, max_interactions=2_000_000_000,
                          late_after=late_after, mrw_eager_after=late_after)
    return descs, dust, opts


def _rho(models, dev):
    return torch.as_tensor(np.concatenate([thermal.stack_density(m.grid).reshape(-1)
                                           for m in models]), device=dev)


def _workspace_run(L, models, descs, dust, opts, rho, stream, dev):
    """pdgpu_mctherm with a caller-allocated workspace: the expected result."""
    nbytes = L.pdgpu_mctherm_workspace_bytes(len(models), descs, C.byref(dust), C.byref(opts))
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    T = torch.empty(rho.numel(), dtype=torch.float64, device=dev)
    st = _lib.McStats()
    assert L.pdgpu_mctherm(len(models), descs, C.byref(dust), C.byref(opts), rho.data_ptr(),
                           T.data_ptr(), ws.data_ptr(), nbytes, stream, C.byref(st)) == 0
    return T, st


def _static_run(L, models, descs, dust, opts, rho, stream, dev):
    T = torch.full((rho.numel(),), -1.0, dtype=torch.float64, device=dev)
    st = _lib.McStats()
    rc = L.pdgpu_mctherm_static(len(models), descs, C.byref(dust), C.byref(opts),
                                rho.data_ptr(), T.data_ptr(), stream, C.byref(st))
    assert rc == 0, _lib.STATUS.get(rc)
    torch.cuda.synchronize(dev)
    return T, st


def test_static_entry_point_matches_workspace_entry_point(cuda):
    """Two static calls of one workload with a different workload between them (three
    models, another packet count and park limit, so its tables, queues and parked packets
    reach past the first workload's offsets): each call equals pdgpu_mctherm bit for bit."""
    L = _lib.lib()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    keep = []
    models_a = workloads.walker_models(n=2, seed=3, scale=0.12)
    a = _descriptors(models_a, 6000, keep)
    rho_a = _rho(models_a, cuda)
    models_b = workloads.walker_models(n=3, seed=9, scale=0.18)
    b = _descriptors(models_b, 9000, keep, late_after=80, seed=17)
    rho_b = _rho(models_b, cuda)
    T_a, st_a = _workspace_run(L, models_a, *a, rho_a, stream, cuda)
    T_b, st_b = _workspace_run(L, models_b, *b, rho_b, stream, cuda)
    assert st_a.parked > 0 and st_b.parked > 0   # the continuation path runs too
    assert rho_b.numel() > rho_a.numel()
    for call, (models, d, rho, T_ref, st_ref) in enumerate(
            [(models_a, a, rho_a, T_a, st_a), (models_b, b, rho_b, T_b, st_b),
             (models_a, a, rho_a, T_a, st_a)]):
        T, st = _static_run(L, models, *d, rho, stream, cuda)
        assert torch.equal(T, T_ref), call
        # every counter of the walk; "drained" counts how many resumed packets were handed
        # to the one-per-warp stage, which depends on timing, not on the result
        got, want = st.asdict(), st_ref.asdict()
        got.pop("drained"), want.pop("drained")
        assert got == want, call


def test_static_entry_point_rejects_runs_beyond_its_scratch(cuda):
    L = _lib.lib()
    big = workloads.small_disk(nr=24, ntheta=24, mass=1e-5)
    keep = []
    # the parking buffer alone (one 128-byte record per 128 packets) exceeds 32 MiB
    descs, dust, opts = _descriptors([big], 50_000_000, keep)
    nbytes = L.pdgpu_mctherm_workspace_bytes(1, descs, C.byref(dust), C.byref(opts))
    assert nbytes > 32 << 20
    T = torch.empty(1, dtype=torch.float64, device=cuda)
    rc = L.pdgpu_mctherm_static(1, descs, C.byref(dust), C.byref(opts), T.data_ptr(),
                                T.data_ptr(), torch.cuda.current_stream(cuda).cuda_stream, None)
    assert rc == 9 and L.pdgpu_status_string(rc) == b"run needs more than the library's static scratch"
