"""amca_plain_run_noalloc: the plain-realm run for callers that cannot let the
library allocate device memory (for example a coupled solver that has
reserved the GPU's memory for its own pool). The caller owns every input and
output buffer; the run's scratch lives in the library's static device array.

Checked here through the C ABI against the ordinary entry point
(amca_create/amca_initialize/amca_run), bit for bit, on two calls in a row
(the static array keeps the previous call's contents, so the second call
shows that everything that must start at zero is cleared).
"""
import ctypes
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def l2g_of(euler: np.ndarray) -> np.ndarray:
    """Local->global matrices with the host libm (Python's math calls it),
    in the reference's operation order (CA/src/Octahedron.cpp:282-310)."""
    out = np.empty((len(euler), 9), np.float64)
    for k, (a, b, g) in enumerate(euler.tolist()):
        ca, sa, cb, sb, cg, sg = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(g), math.sin(g)
        out[k] = [ca * cg - sa * cb * sg, -ca * sg - sa * cb * cg, sa * sb,
                  sa * cg + ca * cb * sg, -sa * sg + ca * cb * cg, -ca * sb,
                  sb * sg, sb * cg, cb]
    return out


def test_noalloc_run_matches_the_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import amca3d_gb300 as A

    lib = A.load_library()
    case = [c for c in cases.small_cases() if c.name == "mixed_24_s1"][0]

    # the ordinary entry point
    realm = A.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    realm.initialize()
    realm.run()
    want = realm.field("orientation_id")
    want_stats = realm.stats()
    realm.close()

    # inputs prepared on the host, copied into device buffers the caller owns
    prep = A.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    prep.prepare()
    site_cells, site_dtc = prep.sites()
    l2g = l2g_of(prep.orientations(all=True))
    prep.close()
    dev = torch.device("cuda", 0)
    d_cells = torch.from_numpy(site_cells).to(dev)
    d_dtc = torch.from_numpy(site_dtc).to(dev)
    d_l2g = torch.from_numpy(l2g).to(dev)
    d_orient = torch.full((case.n_ghost,), 7, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()

    p = A.PlainParams(case.cells[0], case.cells[1], case.cells[2], case.origin[0], case.origin[1], case.origin[2],
                      case.cell_size, case.initial_temperature, case.melting_temperature, case.t_dot, case.a[0],
                      case.a[1], case.a[2], case.time_step, case.termination_time,
                      0.2 if case.time_step_factor_ca is None else case.time_step_factor_ca, case.trunc_coeff())
    golden = np.load(os.path.join(ROOT, "tests", "golden", "mixed_24_s1.npz"))
    for call in range(2):
        res = A.PlainResult()
        err = ctypes.create_string_buffer(256)
        rc = lib.amca_plain_run_noalloc(0, ctypes.byref(p), d_cells.data_ptr(), d_dtc.data_ptr(), len(site_cells),
                                        d_l2g.data_ptr(), d_orient.data_ptr(), -1, None, ctypes.byref(res), err, 256)
        assert rc == 0, err.value.decode()
        got = d_orient.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}"
        # and the unmodified reference's own field for this deck
        assert np.array_equal(got, golden["orient"]), f"call {call}"
        assert res.steps == int(golden["steps"]) == want_stats["step"] and res.done == 1
        assert res.grains == want_stats["grains"] and res.orientations == want_stats["orientations"]


def test_noalloc_rejects_a_bad_site_list():
    """A site cell outside the grid's interior, or out of ascending order, is
    refused before any kernel indexes the field with it."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import amca3d_gb300 as A

    lib = A.load_library()
    case = [c for c in cases.small_cases() if c.name == "mixed_24_s1"][0]
    prep = A.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    prep.prepare()
    site_cells, site_dtc = prep.sites()
    l2g = l2g_of(prep.orientations(all=True))
    prep.close()
    p = A.PlainParams(case.cells[0], case.cells[1], case.cells[2], case.origin[0], case.origin[1], case.origin[2],
                      case.cell_size, case.initial_temperature, case.melting_temperature, case.t_dot, case.a[0],
                      case.a[1], case.a[2], case.time_step, case.termination_time,
                      0.2 if case.time_step_factor_ca is None else case.time_step_factor_ca, case.trunc_coeff())
    dev = torch.device("cuda", 0)
    d_dtc = torch.from_numpy(site_dtc).to(dev)
    d_l2g = torch.from_numpy(l2g).to(dev)
    d_orient = torch.full((case.n_ghost,), 7, dtype=torch.int32, device=dev)
    k = len(site_cells) // 2
    for bad_value in (case.n_ghost + 5, -3, 0, int(site_cells[k - 1])):  # past the end, negative, ghost, repeat
        bad = site_cells.copy()
        bad[k] = bad_value
        d_cells = torch.from_numpy(bad).to(dev)
        res = A.PlainResult()
        err = ctypes.create_string_buffer(256)
        rc = lib.amca_plain_run_noalloc(0, ctypes.byref(p), d_cells.data_ptr(), d_dtc.data_ptr(), len(bad),
                                        d_l2g.data_ptr(), d_orient.data_ptr(), -1, None, ctypes.byref(res), err, 256)
        assert rc == -1, (bad_value, rc, err.value)
        assert f"site {k}".encode() in err.value, err.value
        assert bool((d_orient == 7).all().item()), "the field was written although the site list was refused"


def test_noalloc_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import amca3d_gb300 as A

    lib = A.load_library()
    p = A.PlainParams(400, 400, 400, 0, 0, 0, 1e-6, -0.2, 0, -50, 0, 2e-4, 0, 1e-3, 1.0, 0.2, 1.7320508)
    res = A.PlainResult()
    err = ctypes.create_string_buffer(256)
    small = torch.zeros(16, dtype=torch.int32, device="cuda")  # never written: the size check comes first
    rc = lib.amca_plain_run_noalloc(0, ctypes.byref(p), None, None, 0, None, small.data_ptr(), -1, None,
                                    ctypes.byref(res), err, 256)
    assert rc == -1 and b"too large" in err.value
    assert int(small.abs().sum().item()) == 0
