"""Particle frames in the reference's text format (SerializerSaveSphDataSet3 writes them,
SerializerLoadSphDataSet3 reads them).

The oracle's restatements (oracle/sph_oracle.c: orc_frame_text, orc_frame_parse) are pinned
against the reference itself (tests/golden/frame_f32.npz: the bytes its serializer wrote,
the values its reader read, from its own frame and from a frame of awkward lines); the
device writer and reader are compared with both, byte for byte and bit for bit.
"""
import json
import os
import struct

import numpy as np
import pytest

import bubbles_gb300 as bb
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "frame_f32.npz")
PVDM = bb.FRAME_POSITION | bb.FRAME_VELOCITY | bb.FRAME_DENSITY | bb.FRAME_MASS


def bits_equal(a, b):
    """Bitwise equality of float arrays, any NaN matching any NaN (payloads differ by CPU)."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32)))


def golden():
    d = np.load(GOLDEN, allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["scene"]))


def printf_g(f):
    """C printf("%g", (double)f) for a float32 (glibc keeps the sign of a NaN)."""
    f = np.float32(f)
    if np.isnan(f):
        return "-nan" if struct.unpack("<I", struct.pack("<f", f))[0] >> 31 else "nan"
    return "%g" % float(f)


# ---------------------------------------------------------------------------------------
# CPU: the formatter and the oracle
# ---------------------------------------------------------------------------------------
EDGE = [0.0, -0.0, 1.0, -1.0, 0.5, 1e-4, 9.99999e-5, 1e-5, 123456.0, 999999.0, 999999.5,
        9999995.0, 1e6, 1e-6, 0.000100000005, 3.4028235e38, 1.17549435e-38, 1.4e-45,
        1.0e-40, 0.1, 0.2, 0.3, 100.0, 1000.0, 2.5, 0.0625, 16777216.0, 8388607.5, 1e10,
        -7.8125e-3, 1234.5, 12345.65, 0.00792256, np.inf, -np.inf]


def test_format_g_edge_cases(native):
    for v in EDGE:
        assert bb.format_g(v) == printf_g(v), v
    nan = struct.unpack("<f", struct.pack("<I", 0x7FC00000))[0]
    nneg = struct.unpack("<f", struct.pack("<I", 0xFFC00000))[0]
    assert bb.format_g(nan) == "nan"
    assert bb.format_g(nneg) == "-nan"


def test_format_g_random_bit_patterns(native):
    """Every exponent range, subnormals included: random float32 bit patterns."""
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 2**32, size=20000, dtype=np.uint64).astype(np.uint32)
    vals = bits.view(np.float32)
    vals = vals[np.isfinite(vals)]
    bad = [float(v) for v in vals if bb.format_g(float(v)) != printf_g(v)]
    assert not bad, bad[:5]


def test_format_g_rounding_boundaries(native):
    """Values next to the six-digit rounding boundaries (ties go to even on the exact
    binary value, carries move the decimal exponent)."""
    base = np.array([9.999995, 99999.95, 0.00999999, 1.000005, 0.000123456, 5e-5, 99999.5,
                     999999.5, 9.5, 0.95, 1.5e-5], np.float32)
    for b in base:
        for k in range(-4, 5):
            x = b
            toward = np.float32(np.inf) if k > 0 else np.float32(-np.inf)
            for _ in range(abs(k)):
                x = np.nextafter(x, toward, dtype=np.float32)
            assert bb.format_g(float(x)) == printf_g(x), float(x)


def test_oracle_frame_is_the_reference_serializer():
    """The oracle's frame text equals the bytes SerializerSaveSphDataSet3 wrote (FP32 build)."""
    g, sc = golden()
    t = O.frame_text(g["step3_pos"], g["step3_vel"], g["step3_density"], float(g["mass"]),
                     sc["spacing"], PVDM)
    assert t == g["frame_pvdm"].tobytes()
    assert O.frame_text(g["step3_pos"], spacing=sc["spacing"], flags=bb.FRAME_POSITION) == g["frame_p"].tobytes()


def test_host_formatter_reproduces_reference_lines(native):
    """Lines built from the device formatter's code (run on the host) equal the reference's."""
    g, _ = golden()
    ref = g["frame_pvdm"].tobytes().decode().split("\n")
    start = ref.index("\tDataBegin") + 1
    p, v, r = (np.asarray(g[k], np.float32) for k in ("step3_pos", "step3_vel", "step3_density"))
    m = np.float32(g["mass"])
    for i in range(0, len(p), 7):
        fields = [bb.format_g(float(x)) for x in (*p[i], *v[i], r[i], m)]
        assert "\t\t" + " ".join(fields) == ref[start + i], i


def test_oracle_reader_is_the_reference_reader():
    """The oracle's SerializerLoadParticles3 restatement reads what the reference read, from
    a frame it wrote and from the hand-written frame of awkward lines."""
    g, _ = golden()
    fl, cnt, p, v, d, _ = O.frame_parse(g["frame_pvdm"].tobytes())
    assert fl == int(g["load_pvdm_flags"]) == PVDM and cnt == len(p) == 1440
    assert bits_equal(p, g["load_pvdm_pos"]) and bits_equal(v, g["load_pvdm_vel"])
    assert bits_equal(d, g["load_pvdm_density"])
    fl, cnt, p, v, _, _ = O.frame_parse(g["awkward_frame"].tobytes())
    assert fl == int(g["awkward_flags"]) and cnt == len(p) == 10
    assert bits_equal(p, g["awkward_pos"]) and bits_equal(v, g["awkward_vel"])


def test_section_finder(native):
    g, _ = golden()
    text = g["awkward_frame"].tobytes()
    fl, cnt, a, b = bb.frame_section(text)
    assert (fl, cnt) == (3, 10)
    assert text[a:].startswith(b"\t\t0.1 0.2 0.3") and text[b:].startswith(b"\tDataEnd\n")
    assert b"# comment line inside data DataEnd" in text[a:b]   # a comment does not end the data
    two = g["frame_pvdm"].tobytes() + g["frame_p"].tobytes()
    fl, cnt, a, b = bb.frame_section(two)
    assert fl == PVDM and two[b:].startswith(b"\tDataEnd\nFluidEnd\nFluidBegin")   # the first section
    assert bb.frame_section(b"FluidBegin\n\t\"Count\" 2\n\tDataBegin\n\t\t1 2 3\n\tDataEnd\n", 1)[0] == 1
    for bad in (text.replace(b"\tDataEnd", b"\tDataStop"), text.replace(b"DataBegin", b"DataBeg"),
                text.replace(b"FluidBegin", b"FluidStart")):
        with pytest.raises(bb.BbgError):
            bb.frame_section(bad)
    with pytest.raises(bb.BbgError):
        bb.frame_section(text.replace(b"\"Format\" pv", b"\"Format\" pq"))   # unknown letter


# ---------------------------------------------------------------------------------------
# GPU: the device writer
# ---------------------------------------------------------------------------------------
@pytest.mark.gpu
def test_frame_matches_reference_serializer(gpu):
    g, sc = golden()
    with bb.Solver(sc, pos=g["step3_pos"], vel=g["step3_vel"]) as s:
        assert np.float32(s.scalars()["mass"]) == np.float32(g["mass"])
        s.set(bb.FIELD_DENSITY, g["step3_density"])
        assert s.frame_text(PVDM) == g["frame_pvdm"].tobytes()
        assert s.frame_text(bb.FRAME_POSITION) == g["frame_p"].tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [0x01, 0x02, 0x04, 0x20, 0x03, 0x24, 0x27])
def test_frame_of_moving_state(gpu, moved, flags):
    sc, p, v = moved
    with bb.Solver(sc, pos=p, vel=v) as s:
        for _ in range(3):
            s.advance_time_step(sc["dt"])
        pos, vel = s.download()
        rho = s.get(bb.FIELD_DENSITY)
        mass = s.scalars()["mass"]
        want = O.frame_text(pos, vel, rho, mass, sc["spacing"], flags)
        assert s.frame_text(flags) == want


@pytest.mark.gpu
def test_frame_append_and_errors(gpu, small, tmp_path):
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        # a new particle set has zero densities, as the reference's
        fresh = s.frame_text(bb.FRAME_DENSITY).split(b"\tDataBegin\n")[1].split(b"\tDataEnd")[0]
        assert fresh == b"\t\t0\n" * len(pos)
        for bad in (0, 0x08, 0x10, 0x100, 0x01 | 0x40):
            with pytest.raises(bb.BbgError):
                s.frame_text(bad)
        s.advance_time_step(sc["dt"])
        text = s.frame_text(PVDM)
        path = tmp_path / "frames.txt"
        s.frame_append(path, PVDM)
        s.frame_append(path, PVDM)
        assert path.read_bytes() == text + text
        assert text.startswith(b"FluidBegin\n\t\"Type\" particles\n\t\"Count\" %d\n\t\"Format\" pvdm\n"
                               % len(pos))
        assert text.endswith(b"\tDataEnd\nFluidEnd\n")


@pytest.mark.gpu
def test_frame_full_size_1m(gpu):
    """1,048,576 particles in motion: the device frame equals the oracle's byte for byte."""
    sc, pos = bb.scenes.pcisph_1m()
    with bb.Solver(sc, pos=pos) as s:
        for _ in range(5):
            s.advance_time_step(sc["dt"])
        p, v = s.download()
        rho = s.get(bb.FIELD_DENSITY)
        text = s.frame_text(PVDM)
        want = O.frame_text(p, v, rho, s.scalars()["mass"], sc["spacing"], PVDM)
        assert len(text) == len(want)
        assert text == want


# ---------------------------------------------------------------------------------------
# GPU: the device reader
# ---------------------------------------------------------------------------------------
@pytest.mark.gpu
def test_frame_load_matches_reference_reader(gpu):
    g, sc = golden()
    with bb.Solver(sc, capacity=1440) as s:
        assert s.frame_load(g["frame_pvdm"].tobytes()) == PVDM
        p, v = s.download()
        assert s.n == 1440
        assert bits_equal(p, g["load_pvdm_pos"]) and bits_equal(v, g["load_pvdm_vel"])
    with bb.Solver(sc, capacity=16) as s:
        assert s.frame_load(g["awkward_frame"].tobytes()) == int(g["awkward_flags"])
        p, v = s.download()
        assert bits_equal(p, g["awkward_pos"]) and bits_equal(v, g["awkward_vel"])


@pytest.mark.gpu
def test_frame_load_full_size_round_trip(gpu, tmp_path):
    """1,048,576 particles in motion: frame written on the device, appended twice to a file,
    read back on the device from the file's first section; equal to the oracle's reading,
    and within the six printed digits of the state."""
    sc, pos = bb.scenes.pcisph_1m()
    with bb.Solver(sc, pos=pos) as s:
        for _ in range(3):
            s.advance_time_step(sc["dt"])
        p0, v0 = s.download()
        text = s.frame_text(PVDM)
        path = tmp_path / "frames.txt"
        s.frame_append(path, PVDM)
        s.frame_append(path, PVDM)
    fl, cnt, pw, vw, _, _ = O.frame_parse(text)
    assert cnt == len(pw) == len(pos)
    with bb.Solver(sc, capacity=len(pos)) as r:
        assert r.frame_load(path) == PVDM
        p, v = r.download()
    assert bits_equal(p, pw) and bits_equal(v, vw)
    assert np.all(np.abs(p - p0) <= 5.2e-6 * np.maximum(np.abs(p0), 1e-30))   # six digits
    assert np.all(np.abs(v - v0) <= 5.2e-6 * np.maximum(np.abs(v0), 1e-30))


@pytest.mark.gpu
def test_frame_load_refusals(gpu, small):
    sc, pos = small
    g, _ = golden()
    text = g["frame_pvdm"].tobytes()
    with bb.Solver(sc, pos=pos[:100], capacity=1440) as s:
        before = s.download()
        for bad in (text.replace(b"\tDataEnd", b"\tDataStop"),            # unterminated
                    text.replace(b"\"Count\" 1440", b"\"Count\" 1441"),   # fewer lines than Count
                    text.replace(b"\"Format\" pvdm", b"\"Format\" pvdq")):  # unknown letter
            with pytest.raises(bb.BbgError):
                s.frame_load(bad)
            after = s.download()
            assert np.array_equal(before[0], after[0])
    with bb.Solver(sc, capacity=1000) as s:
        with pytest.raises(bb.BbgError):
            s.frame_load(text)   # capacity

