"""Host logic and the C ABI, without a GPU: the library builds, loads and
exports every function include/mcd.h declares; struct layouts agree; the
host-only entry points (material constants) and the host grid search match
the reference's golden values; the input.file parser keeps its semantics."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mcd import _lib, config, tables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mcd.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mcd_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = declared_functions()
    assert "mcd_run" in names and "mcd_build_table" in names
    for name in names:
        assert hasattr(L, name), name
        assert name in _lib.SIGNATURES, "no ctypes signature for " + name


def test_struct_layouts_match():
    L = _lib.lib()
    for name, cls in _lib.STRUCTS.items():
        assert L.mcd_struct_size(name.encode()) == C.sizeof(cls), name
    assert C.sizeof(_lib.Event) == 40


def test_abi_and_errors():
    L = _lib.lib()
    assert L.mcd_abi_version() == _lib.ABI_VERSION == 10
    assert L.mcd_strerror(_lib.EINVAL) == b"invalid argument"
    m = _lib.Material()
    assert L.mcd_material_init(b"Fe", C.byref(m)) == _lib.ENOSPECIES
    assert L.mcd_material_init(None, C.byref(m)) == _lib.EINVAL


def test_entry_points_reject_bad_arguments_without_touching_the_gpu():
    L = _lib.lib()
    assert L.mcd_run(None, None, None, None, None, None, None, None, 128, None) == _lib.EINVAL
    assert L.mcd_batch_workspace_bytes(0) == 0
    assert L.mcd_batch_workspace_bytes(257) == 0
    assert L.mcd_batch_upload_bytes(0) == 0 and L.mcd_batch_upload_bytes(257) == 0
    # the upload is the workspace less its 64 table slots (4096 x 12 floats each)
    assert L.mcd_batch_upload_bytes(64) <= L.mcd_batch_workspace_bytes(64) - 64 * 4 * 4096 * 12
    assert L.mcd_build_table(0, None, 0, 1, 2, None, None, None, None, None, None, None) == _lib.EINVAL
    assert L.mcd_run_batched(None, 1, None, None, None, None) == _lib.EINVAL


@pytest.mark.parametrize("sp", ["Al", "Si", "Cu", "Au"])
def test_material_constants(golden, sp):
    m = _lib.material(sp)
    ref = golden["physics"][sp + "/const"]
    got = np.array([m.atnd, m.plasmon_e, m.fermi_e])
    assert np.max(np.abs(got - ref) / ref) < 1e-14
    assert m.species.decode() == sp
    assert m.n_shells == {"Al": 3, "Si": 3, "Cu": 4, "Au": 8}[sp]


def test_grid_search_matches_reference(golden):
    """The host grid search picks the reference's exact float32 W and E grids
    for every table of the benchmark configurations."""
    T = golden["tables"]
    for key in T["names"]:
        sp = str(T[key + "/species"])
        kind = key.split("/")[1]
        E0, Emin, Wc, tol = T[key + "/spec"]
        Ws, Es = tables.find_grids(kind, _lib.material(sp), E0, Emin, Wc, tol, tol)
        assert np.array_equal(Ws, T[key + "/Ws"]), key
        assert np.array_equal(Es, T[key + "/Es"]), key


def test_grid_search_fails_like_reference_for_deep_shells():
    """Si 1s at tol 1e-3 has no grid within 1e6 points (the reference raises
    StopIteration); the library raises TableBuildError."""
    m = _lib.material("Si")
    spec = tables._Spec("Gryz", m, 10000.0, 1000.0, 100.0, 1e-3, 1e-3)
    spec.Wmin = spec.Eb = 1189.0
    spec.nfree = 2.0
    spec.Emin = 1189.0
    with pytest.raises(tables.TableBuildError):
        Ws = tables.find_W_series(spec)
        tables.find_E_series(spec, Ws)


INPUT = """# a test input file
num_el   : 64 #multiples of 4
E0       : 15000 # eV
Emin     : 1000
material : Al
s_tilt   : 70
thickness :  5e5
elastic  : Ruth_vanilla
mode     : cont
Bethe_model : JL
diffMFP    : no
gen_tables : yes
tol_E : 1e-3
tol_W : 1e-3
maxScatt: 100000
Wc       : 100
electron_output : outcome, final_E, final_dir
scatter_output : type, E_loss,pathl
"""


def test_input_parser(tmp_path):
    f = tmp_path / "input.file"
    f.write_text(INPUT)
    p = config.readInput(str(f))
    assert p["num_el"] == 64 and isinstance(p["num_el"], int)
    assert p["E0"] == 15000.0 and isinstance(p["E0"], float)
    assert p["material"] == "Al" and p["mode"] == "cont" and p["Bethe_model"] == "JL"
    assert p["diffMFP"] is False and p["gen_tables"] is True
    assert p["electron_output"] == ["outcome", "final_E", "final_dir"]
    assert p["scatter_output"] == ["type", "E_loss", "pathl"]
    assert p["thickness"] == 5e5 and p["maxScatt"] == 100000
    q = config.with_defaults({"E0": 1.0})
    assert q["E0"] == 1.0 and q["thickness"] == 1e30


def test_elastic_dispatch_follows_reference_string_tests():
    from mcd import engine
    DS, CONT = _lib.MODE_DS, _lib.MODE_CONT
    # DS: exact names, and the wDefl-vanilla branch that calls an unimported function
    assert engine.elastic_model("Ruth_vanilla", DS) == _lib.ELASTIC_RUTH
    assert engine.elastic_model("Ruth_nigram", DS) == _lib.ELASTIC_NIGRAM
    assert engine.elastic_model("Ruth_nigram_wDefl", DS) == _lib.ELASTIC_NIGRAM_WDEFL
    with pytest.raises(NameError):
        engine.elastic_model("Ruth_vanilla_wDefl", DS)
    # continuous: substring tests, wDefl variants fall back to the base model
    assert engine.elastic_model("Ruth_vanilla_wDefl", CONT) == _lib.ELASTIC_RUTH
    assert engine.elastic_model("Ruth_nigram_wDefl", CONT) == _lib.ELASTIC_NIGRAM
    # one-to-one mapping on request
    for name, code in _lib.ELASTIC.items():
        assert engine.elastic_model(name, DS, "intended") == code
        assert engine.elastic_model(name, CONT, "intended") == code
    with pytest.raises(NotImplementedError):
        engine.elastic_model("Mott", DS)
    with pytest.raises(ValueError):
        engine.elastic_model("Ruth_other", DS)


def test_diffraction_needs_extinction_distance():
    from mcd import engine
    p = config.parse_input(INPUT)
    p.update(mode="DS", material="Si", diffMFP=True, thickness=3000.0)
    s = engine.make_sim(p, 16)
    assert s.diff_mfp == 1 and s.thickness == 3000.0
    assert _lib.material("Si").xip_g == 1360.0
    with pytest.raises(KeyError):
        engine.make_sim(dict(p, material="Al"), 16)
    # continuous mode has no diffraction channel (MC/tools/scattering.py:753-800)
    assert engine.make_sim(dict(p, mode="cont"), 16).diff_mfp == 0


def test_sim_struct_from_input():
    from mcd import engine
    p = config.parse_input(INPUT)
    s = engine.make_sim(p, 64, seed=3)
    assert s.mode == _lib.MODE_CONT and s.bethe_model == _lib.BETHE["JL"]
    assert s.num_el == 64 and s.seed == 3 and s.s_tilt == 70.0
    with pytest.raises(NotImplementedError):
        engine.make_sim(dict(p, elastic="Mott"), 1)


def test_new_fields_are_validated_before_any_gpu_work():
    """Elastic model codes, the diffraction switch and the adjoint's quantity
    are checked on the host: a bad value returns MCD_EINVAL before a launch."""
    from mcd import engine
    L = _lib.lib()
    p = config.parse_input(INPUT)
    mat = _lib.material("Al")
    s = engine.make_sim(p, 16)                       # continuous mode, Al
    s.elastic = 7
    assert L.mcd_run(C.byref(s), C.byref(mat), None, None, 1, None, None, 1, 128, None) == _lib.EINVAL
    s = engine.make_sim(p, 16)
    s.diff_mfp = 1                                   # continuous mode has no diffraction channel
    assert L.mcd_run(C.byref(s), C.byref(mat), None, None, 1, None, None, 1, 128, None) == _lib.EINVAL
    h = _lib.SoftHist(64, 5, 0.0, 1.0, 0.1)          # unknown quantity
    buf = _lib.AdjointBuf(1, 1, 1, 4, 0)
    assert L.mcd_adjoint_forward(C.byref(engine.make_sim(p, 16)), C.byref(mat), C.byref(h), C.byref(buf), 1, None,
                                 1, None) == _lib.EINVAL
    assert L.mcd_project_detector(None, 5, _lib.FP32, 20.0, 0.0, 0.0, 0.0, None, None) == _lib.EINVAL
    # a cross-section table is for DS FP32 transport only
    s = engine.make_sim(p, 16)                       # continuous mode
    s.sigma_table = C.addressof(C.c_float(0.0))
    assert L.mcd_run(C.byref(s), C.byref(mat), None, None, 1, None, None, 1, 128, None) == _lib.EINVAL
    assert L.mcd_build_sigma_table(C.byref(s), C.byref(mat), None, None) == _lib.EINVAL
    assert L.mcd_sigma_table_bytes() == 1 << 20
    # an FP64 table covers whole octaves of (Emin, E0]: 10 eV to 30 keV for
    # Au (twelve octaves of 256 cells x 46 doubles) exceeds the buffer; the
    # size is checked before any launch
    au = _lib.material("Au")
    assert 8 * 12 * 256 * tables.sig64_stride(au.n_shells + 3) > L.mcd_sigma_table_bytes()
    assert 8 * 10 * 256 * tables.sig64_stride(au.n_shells + 3) <= L.mcd_sigma_table_bytes()   # from 50 eV
    s = engine.make_sim(dict(material="Au", E0=30000.0, Emin=10.0, Wc=50.0, mode="DS"), 16, precision=_lib.FP64)
    tbl = (C.c_double * 4)()
    addr = (C.addressof(tbl) + 15) & ~15            # 16-byte aligned, as the entry point requires
    assert L.mcd_build_sigma_table(C.byref(s), C.byref(au), C.c_void_p(addr), None) == _lib.ETOOBIG
    s.sigma_table = addr
    assert L.mcd_run(C.byref(s), C.byref(au), None, None, 1, None, None, 1, 128, None) == _lib.ETOOBIG
    # the reserved tuning word must be zero (host buffers: nothing is dereferenced)
    host = (C.c_uint8 * 64)()
    t = _lib.Tune(256, 0, 1, 0, 5)
    assert L.mcd_run_batched(C.cast(host, C.c_void_p), 1, C.cast(host, C.c_void_p), C.byref(t),
                             C.cast(host, C.c_void_p), None) == _lib.EINVAL
    # the 56-register kernel (variant bit 0) runs two blocks of at most 576 threads
    t = _lib.Tune(640, 0, 1, 1, 0)
    assert L.mcd_run_batched(C.cast(host, C.c_void_p), 1, C.cast(host, C.c_void_p), C.byref(t),
                             C.cast(host, C.c_void_p), None) == _lib.EINVAL
    # a packed ring header holds electron indices below 2^28
    s = engine.make_sim(p, 2 ** 28 + 1)
    ring = _lib.EventRing(C.cast(host, C.c_void_p), 1, C.cast(host, C.c_void_p), _lib.EV_PACKED_HEAD, 0)
    assert L.mcd_run(C.byref(s), C.byref(mat), None, None, 1, None, C.byref(ring), 1, 128, None) == _lib.EINVAL
    # ring field bits beyond the columns and the packed header
    ring = _lib.EventRing(C.cast(host, C.c_void_p), 1, C.cast(host, C.c_void_p), 0x80, 0)
    assert L.mcd_run_batched_ring(C.cast(host, C.c_void_p), 1, C.cast(host, C.c_void_p), None, C.byref(ring),
                                  C.cast(host, C.c_void_p), None) == _lib.EINVAL


def test_event_record_sizes_agree_with_library():
    from mcd import engine
    L = _lib.lib()
    assert L.mcd_event_bytes(0) == 40 == L.mcd_event_bytes(_lib.EV_ALL) == C.sizeof(_lib.Event)
    for mask in range(128):   # the columns, with and without the packed header
        assert engine.event_dtype(mask).itemsize == L.mcd_event_bytes(mask), mask
    assert L.mcd_event_bytes(_lib.EV_PATHL | _lib.EV_W | _lib.EV_C2 | _lib.EV_POS | _lib.EV_PACKED_HEAD) == 28
    cfg = _lib.EV_PATHL | _lib.EV_W | _lib.EV_C2 | _lib.EV_POS
    assert L.mcd_event_bytes(cfg) == 32
    assert engine.event_dtype(cfg).names == ("electron", "step_chan", "W", "pathl", "c2", "x", "y", "z")


def test_packed_header_records_unpack_in_ring_order():
    """The event index of a packed-header record is its rank among the
    records of its electron in ring order."""
    from mcd import engine
    fields = _lib.EV_W | _lib.EV_PACKED_HEAD
    dt = engine.event_dtype(fields)
    assert dt.names == ("head", "W")
    # three electrons interleaved in the ring; W = 10 * electron + event
    ring = [(7, 0, 1), (2, 0, 0), (7, 1, 2), (5, 0, 3), (2, 1, 1), (7, 2, 0), (5, 1, 2)]
    rec = np.array([((e << 4) | ch, 10.0 * e + k) for e, k, ch in ring], dtype=dt)
    u = engine.unpack_events(rec, fields)
    assert u.dtype.names == ("electron", "step_chan", "W")
    assert list(u["electron"]) == [2, 2, 5, 5, 7, 7, 7]
    assert list(u["step_chan"] >> 5) == [0, 1, 0, 1, 0, 1, 2]
    assert np.array_equal(u["W"], 10.0 * u["electron"] + (u["step_chan"] >> 5))
    assert list(u["step_chan"] & 31) == [0, 1, 3, 2, 1, 2, 0]
    empty = engine.unpack_events(np.zeros(0, dtype=dt), fields)
    assert empty.size == 0 and empty.dtype.names == ("electron", "step_chan", "W")


def test_c_caller_links_and_runs(tmp_path):
    """The header compiles as strict C99 and a C program links against the
    library and calls its host-only entry points (no GPU call)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = _lib.lib()._name
    exe = str(tmp_path / "capi_check")
    src = os.path.join(ROOT, "tests", "capi_check.c")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        src, lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok %d" % _lib.ABI_VERSION, (r.returncode, r.stdout)


@pytest.mark.parametrize("species", ["Al", "Si", "Cu", "Au"])
def test_fp64_table_size_rule_matches_the_library(species):
    """mcd.tables.sigma_table_fits (which decides whether an FP64 run reads
    a table) and the library's size check agree on both sides of the
    buffer's limit: mcd_run refuses a table that does not fit with
    MCD_ETOOBIG before any launch, and otherwise goes on to the next check
    (here the missing loss tables: MCD_EINVAL)."""
    from mcd import engine
    L = _lib.lib()
    mat = _lib.material(species)
    buf = (C.c_double * 4)()
    addr = (C.addressof(buf) + 15) & ~15
    seen = set()
    for Emin in (1.0, 5.0, 10.0, 30.0, 50.0, 100.0, 500.0, 1000.0):
        for E0 in (5000.0, 10000.0, 30000.0, 60000.0, 1e6):
            s = engine.make_sim(dict(material=species, E0=E0, Emin=Emin, Wc=50.0, mode="DS"), 16,
                                precision=_lib.FP64)
            s.sigma_table = addr
            rc = L.mcd_run(C.byref(s), C.byref(mat), None, None, 1, None, None, 1, 128, None)
            fits = tables.sigma_table_fits(s, mat)
            assert rc == (_lib.EINVAL if fits else _lib.ETOOBIG), (species, Emin, E0, rc)
            seen.add(fits)
    assert seen == {True, False}
