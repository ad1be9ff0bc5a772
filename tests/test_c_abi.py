"""CPU-side checks of the C ABI: the library loads, exports every entry point that
include/nbh.h declares, and its host-only parts (pool sizing, generators, .universe I/O,
argument validation) behave; no CUDA computation is called."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import nbh
from nbh import _lib as L
from nbh import universe as U

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nbh.h")


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nbh_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(L.LIB_PATH)
    names = _declared()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(L.SIGNATURES), set(names) - set(L.SIGNATURES)


def test_config_struct_layout_matches_header():
    cfg = L.NbhConfig()
    L.load().nbh_config_default(C.byref(cfg))
    assert cfg.abi_version == L.NBH_ABI_VERSION
    assert (cfg.theta, cfg.G, cfg.pool_factor) == (0.5, 1.0, 2.0)
    assert cfg.eps == pytest.approx(0.05) and cfg.dt == pytest.approx(0.025)
    assert cfg.vote_width == 64 and cfg.arith == L.NBH_ARITH_FMA and cfg.use_graph == 1
    assert C.sizeof(L.NbhConfig) == 4 * (2 + 7 + 11 + 2)


def test_struct_layouts_match_the_c_compiler(tmp_path):
    """sizeof and field offsets of every struct in include/nbh.h, as gcc lays them out, equal
    the ctypes mirrors the binding uses."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = {"nbh_config": L.NbhConfig, "nbh_stats": L.NbhStats, "nbh_diag": L.NbhDiag, "nbh_tune": L.NbhTune,
               "nbh_host_state": L.NbhHostState}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "nbh.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(out["%s.%s" % (cname, fname)]) == getattr(py, fname).offset, (cname, fname)


def test_java_binding_text_matches_the_structs():
    """The Java FFM binding in INTEGRATION.md lays nbh_config out field by field and allocates
    nbh_tune by size: the field names, their order, the reserved tail and the size equal the
    header's (a stale size would let nbh_autotune write past the Java allocation)."""
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = txt[txt.index("StructLayout CONFIG"):]
    block = block[:block.index(";")]
    names = re.findall(r'JAVA_(?:INT|FLOAT)\.withName\("(\w+)"\)', block)
    fields = [f for f, _ in L.NbhConfig._fields_]
    assert names == fields[:-1] and fields[-1] == "reserved"
    nres = int(re.search(r"sequenceLayout\((\d+), JAVA_INT\)\.withName\(\"reserved\"\)", block).group(1))
    assert nres == getattr(L.NbhConfig, "reserved").size // 4
    assert [int(v) for v in re.findall(r"arena\.allocate\((\d+), 4\)", txt)] == [C.sizeof(L.NbhTune)]


def test_mlp_constants_match_header_and_network_shape():
    """NBH_MLP_PARAMS = 12*64 + 64 + 64*64 + 64 + 64 + 1 (W1, b1, W2, b2, W3, b3), the same in
    the header, the binding and the CPU reference of the network."""
    import mlp_ref
    src = open(HEADER).read()
    hdr = int(re.search(r"#define NBH_MLP_PARAMS (\d+)", src).group(1))
    feats = int(re.search(r"#define NBH_MLP_FEATURES (\d+)", src).group(1))
    assert hdr == L.NBH_MLP_PARAMS == mlp_ref.NPARAMS == 12 * 64 + 64 + 64 * 64 + 64 + 64 + 1
    assert feats == L.NBH_MLP_FEATURES == 12


def test_number_of_nodes_matches_reference_formula():
    # GPUBarnesHutNBodySimulation.java:219-227 (maxComputeUnits 16, WARPSIZE 16)
    def ref(n):
        nn = 2 * n
        if nn < 1024 * 16:
            nn = 1024 * 16
        while nn & 15:
            nn += 1
        return nn
    lib = L.load()
    for n in (1, 2, 8, 4096, 8191, 8193, 16384, 1 << 20, 1000003, 4194304):
        assert lib.nbh_number_of_nodes(n, 2.0) == ref(n), n
    assert lib.nbh_number_of_nodes(0, 2.0) == L.NBH_ERR_INVALID


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES") is None and
                    os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_create_without_gpu_fails_loudly():
    with pytest.raises(nbh.NbhError) as ei:
        nbh.Simulation()
    assert ei.value.code in (L.NBH_ERR_NODEVICE, L.NBH_ERR_CUDA)


def test_invalid_config_rejected():
    for kw in ({"eps": 0.0}, {"vote_width": 8}, {"vote_width": 256}, {"theta": -1.0}, {"pool_factor": 0.0},
               {"vote_width": 64, "arith": L.NBH_ARITH_REFERENCE}, {"vote_width": 128, "arith": L.NBH_ARITH_REFERENCE}, {"force_threads": 96}, {"stack_cap": 300},
               {"stack_cap": 60}, {"stack_cap": 100}, {"build_phases": 2}, {"build_phases": 4},
               {"build_buckets": 3}, {"build_buckets": -1}):
        with pytest.raises(nbh.NbhError) as ei:
            nbh.Simulation(**kw)
        assert ei.value.code == L.NBH_ERR_INVALID, kw


def test_generators_deterministic_and_shaped():
    n = 20000
    a = U.PlummerUniverseGenerator(seed=5).arrays(n)
    b = U.PlummerUniverseGenerator(seed=5).arrays(n)
    c = U.PlummerUniverseGenerator(seed=6).arrays(n)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    assert not np.array_equal(a[0], c[0])
    r = np.sqrt(a[0].astype(np.float64) ** 2 + a[1] ** 2 + a[2] ** 2)
    assert abs(np.median(r) - 1.3048) < 0.05          # Plummer half-mass radius 1.305 a
    assert abs(a[6].astype(np.float64).sum() - 1.0) < 1e-4
    v2 = a[3].astype(np.float64) ** 2 + a[4] ** 2 + a[5] ** 2
    ke = 0.5 * (a[6] * v2).sum()
    assert abs(ke - 3 * np.pi / 64) < 0.01             # virial: K = 3 pi G M^2 / (64 a)

    x, y, z, vx, vy, vz, m = U.UniformBallUniverseGenerator(seed=1, vsigma=0.05).arrays(n)
    assert (x.astype(np.float64) ** 2 + y ** 2 + z ** 2).max() <= 1.0 + 1e-6
    assert abs(np.std(vx) - 0.05) < 0.002
    for gen, rad in ((U.SphericalUniverseGenerator(seed=2), 1.0),
                     (U.MonteCarloSphericalUniverseGenerator(seed=2), 1.0),
                     (U.LonLatSphericalUniverseGenerator(seed=2), 5.0)):
        x, y, z, *_ , m = gen.arrays(4096)
        rr = np.sqrt(x.astype(np.float64) ** 2 + y ** 2 + z ** 2)
        np.testing.assert_allclose(rr, rad, rtol=1e-5)
        assert m[0] == np.float32(1.0 / 4096)
    x, y, z, *_ = U.RandomCubicUniverseGenerator(6.0, seed=3).arrays(4096)
    assert x.min() >= -3.0 and x.max() < 3.0

    x, y, z, vx, vy, vz, m = U.DiscGalaxyGenerator(seed=3).arrays(n)
    assert m[0] == np.float32(0.1) and x[0] == 0 and y[0] == 0
    disc = slice(1, 1 + int(0.9 * (n - 1)))
    assert np.median(np.abs(z[disc])) < 0.1
    R = np.sqrt(x[disc].astype(np.float64) ** 2 + y[disc] ** 2)
    assert abs(np.mean(R) - 2.0) < 0.1                  # exponential disc: <R> = 2 rd
    lz = (x[disc] * vy[disc] - y[disc] * vx[disc])
    assert (lz > 0).mean() > 0.95                      # rotating

    x, y, z, vx, vy, vz, m = U.RotatingDiskGalaxyGenerator(1.0, 1.0, 0.5, seed=1).arrays(1000)
    assert m[0] == np.float32(0.5) and np.all(np.abs(z) <= 1 / 16 + 1e-6)


def test_generator_offset_fills_only_its_range():
    x, y, z, vx, vy, vz, m = (np.full(300, 7.0, np.float32) for _ in range(7))
    U.PlummerUniverseGenerator(seed=1).generate(100, 100, x, y, z, vx, vy, vz, m)
    assert (x[:100] == 7).all() and (x[200:] == 7).all() and (x[100:200] != 7).any()


def test_universe_file_round_trip(tmp_path):
    arrs = U.PlummerUniverseGenerator(seed=3).arrays(1000)
    p = tmp_path / "u.universe"
    U.write_universe(p, *arrs)
    raw = p.read_bytes()
    # ObjectOutputStream header, block-data int, then a float[] with its class descriptor
    assert raw[:6] == bytes([0xAC, 0xED, 0x00, 0x05, 0x77, 0x04])
    assert int.from_bytes(raw[6:10], "big") == 1000
    assert raw[10:16] == bytes([0x75, 0x72, 0x00, 0x02, 0x5B, 0x46])
    assert len(raw) == 10 + 19 + 4 + 6 * (6 + 4) + 7 * 4000
    g = U.SerializedUniverseGenerator(p)
    out = g.arrays(1000)
    for u, v in zip(arrs, out):
        np.testing.assert_array_equal(u, v)
    with pytest.raises(ValueError):
        g.arrays(999)


def test_universe_reader_rejects_garbage(tmp_path):
    p = tmp_path / "bad.universe"
    p.write_bytes(b"\x00" * 100)
    with pytest.raises(nbh.NbhError):
        U.SerializedUniverseGenerator(p)


def _reference_fixture(name):
    import build as B                       # oracle/build.py: NBH_REFERENCE_ROOT or the default
    return os.path.join(B.REFERENCE_ROOT, "universes", name)


@pytest.mark.skipif(not os.path.exists(_reference_fixture("sphericaluniverse1.universe")),
                    reason="reference fixtures not mounted")
def test_reads_reference_universe_fixture():
    """universes/sphericaluniverse1.universe: 32768 bodies on the unit sphere at rest,
    masses 1/32768 (written by UniverseSerializer.java)."""
    g = U.SerializedUniverseGenerator(_reference_fixture("sphericaluniverse1.universe"))
    x, y, z, vx, vy, vz, m = g.arrays(32768)
    r = np.sqrt(x.astype(np.float64) ** 2 + y ** 2 + z ** 2)
    np.testing.assert_allclose(r, 1.0, rtol=1e-5)
    assert (vx == 0).all() and (m == np.float32(1 / 32768)).all()
