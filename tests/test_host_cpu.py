"""Host-side logic on CPU: the C ABI library loads and exports every symbol
that include/gbgrav.h declares, error paths that need no GPU, the seeded
initial conditions, and the State container."""
import ctypes
import importlib
import os
import re

import numpy as np
import pytest

from conftest import PKG_NAME, ROOT, load_golden


def _header_functions():
    src = open(os.path.join(ROOT, "include", "gbgrav.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    b = importlib.import_module(PKG_NAME + "._buildlib")
    if not os.path.exists(b.LIB):
        pytest.skip("libgbgrav.so not built (run __graft_entry__.build())")
    pkg = importlib.import_module(PKG_NAME)
    return pkg.load_library()


def test_library_exports_every_declared_symbol(lib):
    names = _header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(lib):
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    declared = set(_header_functions())
    bound = set(lib_mod.SIGNATURES)
    assert declared == bound, (declared - bound, bound - declared)


def test_null_handles_are_rejected_without_gpu(lib):
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    pkg = importlib.import_module(PKG_NAME)
    with pytest.raises(pkg.GravityError, match="handle is NULL"):
        lib_mod.call("gb_direct_acc", None, None, None, 10, 1.0, 1e-4, 0, None)
    with pytest.raises(pkg.GravityError, match="handle is NULL"):
        lib_mod.call("gb_bh_compute", None, None, None, 10, 0.5, 1e-4, 1.0, 64, 0, None)
    with pytest.raises(pkg.GravityError) as e:
        lib_mod.call("gb_direct_acc_fp64", None, -1, None, 0, 1.0, 1.0, None, None)
    assert e.value.status == lib_mod.GB_EINVAL
    assert lib.gb_version() >= 10000


def test_plummer_sampler_reproduces_reference():
    ic = importlib.import_module(PKG_NAME + ".ic")
    g = load_golden("plummer_ic")
    p, v, m = ic.plummer(1000, 1.0, 1.0, 0, 1.0)
    assert np.array_equal(p, g["pos0"]) and np.array_equal(v, g["vel0"])
    assert np.array_equal(m, g["mass0"])
    p, v, m = ic.plummer(257, 2.5, 0.7, 11, 1.0)
    assert np.array_equal(p, g["pos1"]) and np.array_equal(v, g["vel1"])


def test_disk_and_batch_generators():
    ic = importlib.import_module(PKG_NAME + ".ic")
    p, v, m = ic.exponential_disk(20000, seed=3)
    assert p.shape == (20000, 3) and np.isclose(m.sum(), 5.0)
    R = np.linalg.norm(p[:, :2], axis=1)
    # Exponential surface density: mean radius 2 Rd.
    assert abs(R.mean() / 3.0 - 2.0) < 0.05
    # sech^2 profile: mean |z| = z0 ln 2.
    assert abs(np.abs(p[:, 2]).mean() / 0.3 - np.log(2.0)) < 0.03
    # Net momentum removed.
    assert np.abs((v * m[:, None]).sum(0)).max() < 1e-9
    sizes = ic.batch_sizes(512)
    assert min(sizes) >= 256 and max(sizes) <= 16384
    assert sizes == ic.batch_sizes(512)
    pos, vel, mass = ic.plummer_pair(1000)
    assert pos.shape == (2000, 3)
    assert np.allclose((vel * mass[:, None]).sum(0), 0.0, atol=1e-12)


def test_state_contract():
    pkg = importlib.import_module(PKG_NAME)
    st = pkg.State.from_arrays(np.zeros((5, 3), np.float32), np.ones((5, 3)), np.ones(5))
    assert st.pos.dtype == np.float64 and st.ids.dtype == np.int64
    assert st.ptype.dtype == np.int32 and st.n == 5


def test_potential_struct_layout_and_dict(pkg):
    """gb_potential_t: six doubles then two int32 (56 bytes), filled from the
    engines' `pot` dict."""
    import ctypes
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    ext = importlib.import_module(PKG_NAME + ".solvers.external")
    assert ctypes.sizeof(lib_mod.Potential) == 56
    assert lib_mod.Potential.is_hernquist.offset == 48
    p = ext.Potential.from_dict(dict(M_d=5.0, a=3.0, b=0.3, M_h=12.0, a_h=8.0))
    c = p.to_c()
    assert (c.M_d, c.a, c.b, c.M_h, c.a_h, c.smbh_mass, c.is_hernquist, c.reserved) == \
        (5.0, 3.0, 0.3, 12.0, 8.0, 0.0, 0, 0)
    q = ext.Potential.from_dict(dict(M_d=0.0, a=1.0, b=1.0, M_h=40.0, a_h=15.0, is_hernquist=1,
                                     smbh_mass=0.1))
    assert q.is_hernquist == 1 and q.smbh_mass == 0.1


def test_grid_info_struct_layout():
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    assert ctypes.sizeof(lib_mod.GridInfo) == 72
    assert lib_mod.GridInfo.lo.offset == 32 and lib_mod.GridInfo.inv_cell.offset == 64


def test_diag_struct_layout():
    """gb_diag_t: nine uint64 counters, wait_timeouts last."""
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    assert ctypes.sizeof(lib_mod.Diag) == 72
    assert lib_mod.Diag.wait_timeouts.offset == 64
    assert "wait_timeouts" in lib_mod.Diag().as_dict()


def test_sort_wait_probe_rejects_bad_arguments_without_gpu(lib):
    """gb_sort_wait_probe checks its poll limit and pointers before any CUDA
    call."""
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    pkg = importlib.import_module(PKG_NAME)
    excl = (ctypes.c_uint32 * 256)()
    cnt = ctypes.c_uint64()
    for limit in (0, -5, (1 << 20) + 1):
        with pytest.raises(pkg.GravityError, match="spin_limit") as e:
            lib_mod.call("gb_sort_wait_probe", limit, 0, excl, ctypes.byref(cnt))
        assert e.value.status == lib_mod.GB_EINVAL
    with pytest.raises(pkg.GravityError, match="NULL"):
        lib_mod.call("gb_sort_wait_probe", 10, 0, None, ctypes.byref(cnt))


def test_state_npz_roundtrip(tmp_path):
    st_mod = importlib.import_module(PKG_NAME + ".state")
    rng = np.random.default_rng(3)
    s = st_mod.State.from_arrays(rng.normal(size=(50, 3)), rng.normal(size=(50, 3)), rng.random(50),
                                 time=1.25, step=7, seed=3, u=rng.random(50),
                                 meta={"level": "small", "dt": 1e-3})
    p = str(tmp_path / "snap.npz")
    s.save_npz(p)
    t = st_mod.State.load_npz(p)
    for name in ("pos", "vel", "mass", "ptype", "ids", "u"):
        np.testing.assert_array_equal(getattr(t, name), getattr(s, name))
    assert (t.time, t.step, t.seed) == (1.25, 7, 3)
    assert t.meta["level"] == "small" and t.meta["dt"] == 1e-3 and t.temperature is None


def test_form_selectors_reject_null_handles_without_gpu(lib):
    """The force-pass, band and traversal selectors check their handle before
    any CUDA call."""
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    pkg = importlib.import_module(PKG_NAME)
    for name, args in (("gb_direct_set_variant", (None, 2)), ("gb_direct_set_sym_band", (None, 1 << 30)),
                       ("gb_batch_set_variant", (None, 1)), ("gb_bh_set_traversal", (None, -1)),
                       ("gb_adjoint_set_variant", (None, 2))):
        with pytest.raises(pkg.GravityError, match="handle is NULL"):
            lib_mod.call(name, *args)


def test_python_surface_of_the_force_forms(pkg):
    """Engine(symmetric=...) and diagnostics(), the solver and batch form
    setters, and the autotuner's candidate lists carry the symmetric forms."""
    import inspect
    eng = importlib.import_module(PKG_NAME + ".engine")
    grav = importlib.import_module(PKG_NAME + ".solvers.gravity")
    batch = importlib.import_module(PKG_NAME + ".batch")
    tune = importlib.import_module(PKG_NAME + ".autotune")
    assert inspect.signature(eng.Engine).parameters["symmetric"].default is True
    assert callable(eng.Engine.diagnostics)
    assert callable(grav.DirectGravity.set_variant) and callable(grav.DirectGravity.set_sym_band)
    assert "variant" in inspect.signature(batch.DirectBatch).parameters
    assert (2, 4, 2) in tune.DIRECT_SHAPES and (2, 4, 1) in tune.BATCH_SHAPES


def test_noalloc_rejects_bad_arguments_without_gpu(lib):
    """gb_direct_acc_noalloc refuses flag bits other than GB_ACCUMULATE and
    GB_PLAIN_FP32, and sizes above its static scratch, before any CUDA call
    (the pointers below are never dereferenced)."""
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    pkg = importlib.import_module(PKG_NAME)
    fake = 1 << 12  # aligned, never read
    for bad in (lib_mod.GB_USE_GRAPH, lib_mod.GB_COUNT_WORK, 0x100):
        with pytest.raises(pkg.GravityError, match="flags") as e:
            lib_mod.call("gb_direct_acc_noalloc", fake, fake, 10, 1.0, 1e-4, bad, None)
        assert e.value.status == lib_mod.GB_EINVAL
    with pytest.raises(pkg.GravityError, match="outside") as e:
        lib_mod.call("gb_direct_acc_noalloc", fake, fake, 65537, 1.0, 1e-4, 0, None)
    assert e.value.status == lib_mod.GB_EINVAL


def test_engine_rejects_bad_options_before_touching_the_gpu():
    """Engine's option checks run on the host: precision, fused_potential
    and gravity_mode values outside the documented sets raise ValueError."""
    pkg = importlib.import_module(PKG_NAME)
    for kw in ({"precision": "fp16"}, {"fused_potential": "sometimes"}, {"gravity_mode": "fmm"}):
        with pytest.raises(ValueError):
            pkg.Engine(**kw)
