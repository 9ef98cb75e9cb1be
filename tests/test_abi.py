"""CPU tests of the C ABI: libwavefd.so loads, exports every entry point that
include/wavefd.h declares, and its host-only calls validate their arguments.
No compute call is made (no GPU here)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "wavefd.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wfd_[a-z0-9_]+)\s*\(", text)))


def test_header_declarations_exported():
    from neuralmech_gb300 import _lib
    lib = _lib.load()
    names = _declared()
    assert names, "no declarations parsed"
    for n in names:
        assert hasattr(lib, n), f"{n} declared in wavefd.h but not exported"
    assert set(names) <= set(_lib.EXPORTS) | set(names)
    assert set(_lib.EXPORTS) == set(names)


def test_version_and_strerror():
    from neuralmech_gb300 import _lib
    lib = _lib.load()
    assert lib.wfd_version() >> 16 == 3
    for code in range(0, -8, -1):
        assert lib.wfd_strerror(code).decode()
    assert lib.wfd_strerror(-99).decode() == "unknown status"


def _problem(**kw):
    from neuralmech_gb300 import _lib
    base = dict(ndim=2, order=8, nz=64, ny=1, nx=100, nshot=2, nt=50, nsrc=1, nrec=5,
                ckpt_every=0, ckpt_format=1, lap_store=0, shots_per_cta=0, dt=1e-3, dz=10.0,
                dy=1.0, dx=10.0, src_scale=1.0, vmax=3000.0)
    base.update(kw)
    return _lib.Problem(**base)


def _ws(p, grad=1):
    from neuralmech_gb300 import _lib
    n = ctypes.c_size_t(0)
    rc = _lib.load().wfd_workspace_bytes(ctypes.byref(p), grad, ctypes.byref(n))
    return rc, n.value


def test_update_form_checks_and_workspace():
    """The summed form adds one field (the increment d_n) to the workspace of
    a gradient (auto and summed) or of a forced-summed forward; it is refused
    where only the leapfrog kernels exist."""
    from neuralmech_gb300 import _lib
    field = 2 * 64 * 104 * 4
    _, lf = _ws(_problem(update_form=1), 1)
    _, au = _ws(_problem(update_form=0), 1)
    _, su = _ws(_problem(update_form=2), 1)
    assert au == su and au - lf >= field
    _, f0 = _ws(_problem(update_form=0), 0)
    _, f2 = _ws(_problem(update_form=2), 0)
    assert f2 - f0 >= field
    # two steps per launch: d_n, d_{n+2} and d_{n+1}
    _, l2 = _ws(_problem(update_form=1, step_block=2), 1)
    _, s2 = _ws(_problem(update_form=2, step_block=2), 1)
    assert s2 - l2 >= 3 * field
    # 3D: the summed forward of a gradient adds the increment field too
    _, t1 = _ws(_problem(update_form=1, ndim=3, ny=20, nz=24, nx=40, vmax=2000.0, dy=10.0), 1)
    _, t0 = _ws(_problem(update_form=0, ndim=3, ny=20, nz=24, nx=40, vmax=2000.0, dy=10.0), 1)
    assert t0 - t1 >= 2 * 24 * 20 * 40 * 4
    for bad in (dict(update_form=3), dict(update_form=-1),
                dict(update_form=2, lap_store=2), dict(update_form=2, field_format=1),
                dict(update_form=2, adjoint_mode=1)):
        rc, _ = _ws(_problem(**bad), 0)
        assert rc == _lib.WFD_ERR_INVALID, bad


def test_block_float_levels_workspace_and_checks():
    """WFD_LEVEL_BFP16 keeps the same levels in 2.25 instead of 4 bytes per
    cell; the region also holds the K + 2 FP32 slots of a recomputed segment.
    It needs the two-step summed forward."""
    from neuralmech_gb300 import _lib
    field = 2 * 64 * 104 * 4
    slot = (field + 255) // 256 * 256
    q16 = (2 * 64 * 104 * 2 + 255) // 256 * 256
    e8 = (2 * 64 * 32 + 255) // 256 * 256  # exponent rows of 104 / 4 bytes padded to 32
    kw = dict(nt=100, ckpt_every=10, step_block=2, store_levels=45)  # 4 kept segments: u_60 .. u_99
    rc32, n32 = _ws(_problem(**kw))
    rc16, n16 = _ws(_problem(level_format=1, **kw))
    assert rc32 == 0 and rc16 == 0
    assert n32 - n16 == 42 * slot - 40 * (q16 + e8)
    # the same budget in bytes holds more levels
    from neuralmech_gb300 import Grid, levels_for_budget
    g = Grid((64, 100), (10.0, 10.0), 1e-3, 100)
    b = 10 ** 9
    l32 = levels_for_budget(g, 2, b)
    l16 = levels_for_budget(Grid((64, 100), (10.0, 10.0), 1e-3, 100, level_format="bfp16"), 2, b)
    assert l32 == b // field and l16 == b // (2 * 64 * (2 * 104 + 32))
    assert 1.7 < l16 / l32 < 1.9
    for bad in (dict(level_format=2), dict(level_format=-1), dict(level_format=1),  # step_block 1
                dict(level_format=1, step_block=2, update_form=1),
                dict(level_format=1, step_block=2, lap_store=2),
                dict(level_format=1, step_block=2, field_format=1)):
        rc, _ = _ws(_problem(**bad))
        assert rc == _lib.WFD_ERR_INVALID, bad
    _ws(_problem(level_format=1))
    assert "block-floating-point levels" in _lib.load().wfd_last_error().decode()


def test_workspace_bytes_grows_with_gradient():
    rc0, n0 = _ws(_problem(), 0)
    rc1, n1 = _ws(_problem(), 1)
    assert rc0 == 0 and rc1 == 0 and 0 < n0 < n1
    # two FP32 fields of 2 x 64 x 104 cells at least
    assert n0 >= 2 * 2 * 64 * 104 * 4
    # BF16 checkpoints take about half the FP32 checkpoint space
    _, f32 = _ws(_problem(ckpt_format=0))
    _, b16 = _ws(_problem(ckpt_format=1))
    _, i16 = _ws(_problem(ckpt_format=2))
    assert b16 < i16 < f32


def test_workspace_holds_the_kept_levels():
    """store_levels: the forward keeps the last floor((S - 2) / K) segments'
    levels, u_{k0 - 1} .. u_nt, one FP32 field of nshot x nz x ld each."""
    field = 2 * 64 * 104 * 4
    slot = (field + 255) // 256 * 256
    _, n0 = _ws(_problem(nt=100, ckpt_every=10))
    _, n1 = _ws(_problem(nt=100, ckpt_every=10, store_levels=12))  # = K + 2: the minimum
    _, n4 = _ws(_problem(nt=100, ckpt_every=10, store_levels=45))  # 4 segments: 42 levels
    _, n9 = _ws(_problem(nt=100, ckpt_every=10, store_levels=10 ** 6))  # all 10 segments
    # FP32 checkpoints of the 10 segments: one pair less per kept segment
    ck = 2 * ((field + 255) // 256 * 256)
    _, c0 = _ws(_problem(nt=100, ckpt_every=10, ckpt_format=0))
    _, c4 = _ws(_problem(nt=100, ckpt_every=10, ckpt_format=0, store_levels=45))
    assert n1 == n0
    assert c4 - c0 == (42 - 12) * slot - 3 * ck  # 4 kept segments: the last one kept anyway
    _, c9 = _ws(_problem(nt=100, ckpt_every=10, ckpt_format=0, store_levels=10 ** 6))
    assert c9 - c0 == (102 - 12) * slot - 9 * ck
    # the L u stores (FP32, BF16) do not use it
    _, f0 = _ws(_problem(nt=100, ckpt_every=10, lap_store=2))
    _, f9 = _ws(_problem(nt=100, ckpt_every=10, lap_store=2, store_levels=10 ** 6))
    assert f0 == f9


@pytest.mark.parametrize("bad,code", [
    (dict(ndim=4), -1), (dict(order=6), -1), (dict(ny=3), -1), (dict(nz=8), -1),
    (dict(nshot=0), -1), (dict(nt=0), -1), (dict(dt=0.0), -1), (dict(dx=-1.0), -1),
    (dict(ckpt_format=3), -1), (dict(ckpt_every=-1), -1), (dict(lap_store=3), -1),
    (dict(store_levels=-1), -1), (dict(field_format=3), -1), (dict(field_format=1, ndim=3, ny=64), -1),
    (dict(field_format=2, step_block=2), -1), (dict(adjoint_mode=2), -1),
    (dict(adjoint_mode=1, step_block=2), -1), (dict(adjoint_mode=1, recon_band=40), -1),
    (dict(vmax=1e6), -4),
])
def test_invalid_problems_rejected(bad, code):
    from neuralmech_gb300 import _lib
    rc, _ = _ws(_problem(**bad))
    assert rc == code
    assert _lib.load().wfd_last_error().decode()


def test_cfl_bound_matches_stable_dt():
    from neuralmech_gb300 import stable_dt
    dt = stable_dt((10.0, 10.0), 3000.0, 8)
    assert abs(dt * 3000.0 / 10.0 - 0.5547) < 1e-3
    assert _ws(_problem(dt=dt * 0.999))[0] == 0
    assert _ws(_problem(dt=dt * 1.01))[0] == -4
    dt3 = stable_dt((10.0, 10.0, 10.0), 3000.0, 8)
    assert abs(dt3 * 3000.0 / 10.0 - 0.4529) < 1e-3


def test_null_workspace_and_arguments_rejected():
    from neuralmech_gb300 import _lib
    lib = _lib.load()
    p = _problem()
    assert lib.wfd_forward(ctypes.byref(p), None, None, None, None, None, None, None, None, 0,
                           None, 0, None) == -1
    assert lib.wfd_status(None, None) == -2
    assert lib.wfd_step2d_order2(None, None, None, 1.0, 1.0, 1.0, 1.0, 10, 10, 12, None) == -1
    # misaligned row pitch for the TMA path (M_padded % 4 != 0) is refused before any launch
    buf = ctypes.create_string_buffer(4096 + 16)
    a = ctypes.c_void_p((ctypes.addressof(buf) + 15) // 16 * 16)
    assert lib.wfd_step2d_order2(a, a, a, 1.0, 1.0, 1.0, 1.0, 10, 10, 13, None) == -1


def test_problem_struct_mirrors_header():
    """_lib.Problem has the fields of wfd_problem in the header's order and types."""
    import re
    from neuralmech_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "wavefd.h")).read()
    body = re.search(r"typedef struct wfd_problem \{(.*?)\} wfd_problem;", src, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        fields += [(n.strip(), ctype) for n in names.split(",")]
    mirror = [(n, {ctypes.c_int32: "int32_t", ctypes.c_float: "float"}[t]) for n, t in _lib.Problem._fields_]
    assert mirror == fields


def test_dropin_arguments_rejected():
    """The reduced-precision and 1D drop-ins check their arguments on the host
    (no launch is made here)."""
    from neuralmech_gb300 import _lib
    lib = _lib.load()
    p = ctypes.c_void_p(256)  # never dereferenced: every call below fails its checks first
    assert lib.wfd_step1d(p, p, p, 1.0, 1e-3, 1e-2, 2, None) == -1
    assert lib.wfd_step1d(None, p, p, 1.0, 1e-3, 1e-2, 100, None) == -1
    assert lib.wfd_step2d_mixed(p, p, p, 1.0, 1e-3, 1e-2, 1e-2, 64, 64, 64, None) == -1  # M_padded <= M
    assert lib.wfd_step2d_mixed(p, p, p, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 63, None) == -1  # odd M_padded
    assert lib.wfd_step2d_mixed(ctypes.c_void_p(258), p, p, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 64, None) == -1
    assert lib.wfd_step2d_scaled(p, p, p, p, p, p, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 96, None) == -1  # % 64
    assert lib.wfd_step2d_scaled(ctypes.c_void_p(260), p, p, p, p, p, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 64,
                                 None) == -1  # q not 8-byte aligned
    assert "64" in lib.wfd_last_error().decode() or "aligned" in lib.wfd_last_error().decode()


def test_exact_temporal_and_overlap_arguments_rejected():
    """wfd_step2d_exact, wfd_temporal_step and wfd_misfit_gradient_overlap check
    their arguments on the host (no launch, no device access here)."""
    from neuralmech_gb300 import _lib
    lib = _lib.load()
    p = ctypes.c_void_p(4096)
    q = ctypes.c_void_p(4096 + 64 * 64 * 4)       # a separate 64 x 64 field
    r = ctypes.c_void_p(4096 + 2 * 64 * 64 * 4)
    t = ctypes.c_void_p(4096 + 3 * 64 * 64 * 4)
    assert lib.wfd_step2d_exact(None, p, p, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 64, None) == -1
    assert lib.wfd_step2d_exact(p, p, p, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 59, None) == -1  # M_padded < M
    assert lib.wfd_step2d_exact(p, p, p, 1.0, 1e-3, 1e-2, 1e-2, 2, 60, 64, None) == -1   # N < 3
    assert lib.wfd_temporal_step(p, q, r, t, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 62, None) == -1  # M_padded % 4
    assert lib.wfd_temporal_step(p, q, ctypes.c_void_p(4100), t, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 64,
                                 None) == -1  # v0 not 16-byte aligned
    assert lib.wfd_temporal_step(p, q, p, t, 1.0, 1e-3, 1e-2, 1e-2, 64, 60, 64, None) == -1  # v0 = u0
    assert "overlap" in lib.wfd_last_error().decode()
    assert lib.wfd_temporal_step(p, q, r, ctypes.c_void_p(4096 + 2 * 64 * 64 * 4 + 64), 1.0, 1e-3, 1e-2,
                                 1e-2, 64, 60, 64, None) == -1  # v1 overlaps v0
    pr = _problem()
    assert lib.wfd_misfit_gradient_overlap(ctypes.byref(pr), p, None, None, None, p, p, p, p, None, None,
                                           p, None, p, p, 1 << 20, None) == -1  # no event
    assert "observed_ready" in lib.wfd_last_error().decode()


def test_reduced_precision_fields_halve_the_forward_workspace():
    _, f32 = _ws(_problem(), 0)
    _, f16 = _ws(_problem(field_format=1), 0)
    _, i16 = _ws(_problem(field_format=2), 0)
    field = 2 * 64 * 104 * 4
    assert f32 - f16 >= 2 * field // 2 - 512  # two levels of 2 instead of 4 bytes
    assert f16 < i16 < f32
    rc, _ = _ws(_problem(field_format=1), 1)  # no gradient workspace: forward-only
    assert rc == -1


def test_reconstruction_workspace_keeps_frames_not_checkpoints():
    """adjoint_mode reconstruct: no checkpoints or level slots; the damped
    frame (recon_band cells along every edge) of every level instead."""
    _, ck = _ws(_problem(nt=100, ckpt_every=10, ckpt_format=0))
    _, r0 = _ws(_problem(nt=100, adjoint_mode=1, recon_band=0))
    _, r6 = _ws(_problem(nt=100, adjoint_mode=1, recon_band=6))
    assert r0 < ck and r0 < r6
    # frame of one shot: 2 * 6 full rows of ld = 104 and 52 rows of 8 + (104 - 92) columns
    frame = 2 * (2 * 6 * 104 + (64 - 12) * (8 + 104 - 92)) * 4
    assert r6 - r0 == 101 * ((frame + 255) // 256 * 256)


def test_variable_density_arguments_rejected():
    """The variable-density entries refuse, before any launch: a NULL u_final,
    a 3D problem, and a dt inside the collocated CFL bound but outside the
    staggered operator's (S = 4 (sum|c_k|)^2 = 6.62 at order 8 against 6.50)."""
    from neuralmech_gb300 import _lib, stable_dt
    lib = _lib.load()
    d = ctypes.c_void_p(256)  # never dereferenced: every call fails its host checks
    ws = ctypes.c_size_t(0)

    def final(p, u_final):
        return lib.wfd_vd_forward_final(ctypes.byref(p), d, d, None, None, d, d, d, d, u_final, d, ws, None)

    def forward(p):
        return lib.wfd_vd_forward(ctypes.byref(p), d, d, None, None, d, d, d, d, d, ws, None)

    assert final(_problem(), None) == -1
    assert forward(_problem(ndim=3, ny=8)) == -1
    dt = stable_dt((10.0, 10.0), 3000.0, 8)
    assert _ws(_problem(dt=dt * 0.999))[0] == 0  # the collocated bound holds
    assert forward(_problem(dt=dt * 0.999)) == -4
    assert final(_problem(dt=dt * 0.999), d) == -4


def test_register_window_step_blocks():
    """step_block 8 (order 2) and 4 (order 4): 2D leapfrog FP32 forwards only;
    refused with another order, in 3D, with a gradient, with the summed
    update or reduced-precision fields, and any other value."""
    from neuralmech_gb300 import _lib
    ok = [dict(step_block=8, order=2), dict(step_block=4, order=4)]
    for kw in ok:
        rc, n = _ws(_problem(**kw), 0)
        assert rc == 0 and n > 0, kw
        assert _ws(_problem(**kw), 1)[0] == _lib.WFD_ERR_INVALID, kw  # forward only
        assert _ws(_problem(update_form=2, **kw), 0)[0] == _lib.WFD_ERR_INVALID, kw
        assert _ws(_problem(field_format=1, **kw), 0)[0] == _lib.WFD_ERR_INVALID, kw
    bad = [dict(step_block=8, order=8), dict(step_block=8, order=4), dict(step_block=4, order=2),
           dict(step_block=3, order=2), dict(step_block=16, order=2),
           dict(step_block=8, order=2, ndim=3, ny=20, nz=24, nx=40, vmax=2000.0, dy=10.0)]
    for kw in bad:
        assert _ws(_problem(**kw), 0)[0] == _lib.WFD_ERR_INVALID, kw


def test_batch_plan_arguments_rejected():
    """wfd_batch_plan checks its arguments before any CUDA call."""
    from neuralmech_gb300 import _lib
    lib = _lib.load()
    out = ctypes.c_void_p(123)
    items = (_lib.BatchItem * 2)()
    assert lib.wfd_batch_plan(items, 2, None, None) == _lib.WFD_ERR_INVALID
    assert lib.wfd_batch_plan(None, 2, None, ctypes.byref(out)) == _lib.WFD_ERR_INVALID
    assert out.value is None  # cleared on failure
    assert lib.wfd_batch_plan(items, 0, None, ctypes.byref(out)) == _lib.WFD_ERR_INVALID
    assert lib.wfd_batch_plan(items, 2, None, ctypes.byref(out)) == _lib.WFD_ERR_INVALID  # no problem
    assert "problem" in lib.wfd_last_error().decode()
    assert lib.wfd_batch_run(None, None) == _lib.WFD_ERR_INVALID
    assert lib.wfd_batch_launches(None) == 0
    assert lib.wfd_batch_free(None) == 0

