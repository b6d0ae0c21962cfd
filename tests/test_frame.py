"""Particle frames in the reference's text format (SerializerSaveSphDataSet3).

The oracle's restatement (oracle/sph_oracle.c, orc_frame_text) is pinned against the bytes
the reference serializer itself wrote (tests/golden/frame_f32.npz); the device writer and
its host formatter are compared with both, byte for byte.
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
