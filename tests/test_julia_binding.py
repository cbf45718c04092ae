"""The Julia binding (julia/NQCDGPU.jl) against the C ABI and the engine's
random stream, read as text (no Julia toolchain is needed):

* every C struct of include/nqcd_gpu.h has a Julia mirror with the same
  fields in the same order and the matching Julia types, so that the isbits
  structs have the C layout;
* the enum constants and the ABI version equal the header's;
* the Julia Philox4x32-10 uses the multipliers and Weyl constants of the
  engine (csrc/nqcd_math.h), keys its streams with the engine's stream
  numbers, and its known-answer table equals the oracle's Philox outputs.
"""
import re
from pathlib import Path

import pytest

import oracle as O

ROOT = Path(__file__).resolve().parent.parent
JL = (ROOT / "julia" / "NQCDGPU.jl").read_text()
HEADER = (ROOT / "include" / "nqcd_gpu.h").read_text()
MATH = (ROOT / "nqcdynamics.jl_gb300" / "csrc" / "nqcd_math.h").read_text()

C_TO_JULIA = {
    "int32_t": "Int32",
    "int64_t": "Int64",
    "uint64_t": "UInt64",
    "double": "Float64",
    "float": "Float32",
    "const double*": "Ptr{Float64}",
    "double*": "Ptr{Float64}",
}


def c_struct(name):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), HEADER, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m = re.fullmatch(r"((?:const )?\w+\*?) (.+)", decl)
        ctype, names = m.group(1), m.group(2)
        for n in names.split(","):
            n = n.strip()
            arr = re.fullmatch(r"(\w+)\[(\d+)\]", n)
            if arr:
                fields.append((arr.group(1), f"NTuple{{{arr.group(2)},{C_TO_JULIA[ctype]}}}"))
            elif n.startswith("*"):
                fields.append((n[1:], C_TO_JULIA[ctype + "*"]))
            else:
                fields.append((n, C_TO_JULIA[ctype]))
    return fields


def julia_struct(name):
    body = re.search(r"^struct %s\n(.*?)^end" % name, JL, flags=re.S | re.M).group(1)
    return [tuple(x.strip() for x in line.split("::")) for line in body.strip().splitlines()]


@pytest.mark.parametrize("cname,jname", [("nqcd_config", "NqcdConfig"), ("nqcd_outputs", "NqcdOutputs"),
                                         ("nqcd_stats", "NqcdStats"), ("nqcd_sampler", "NqcdSampler"),
                                         ("nqcd_mapping", "NqcdMapping")])
def test_julia_structs_mirror_the_header(cname, jname):
    c = c_struct(cname)
    j = julia_struct(jname)
    assert [n for n, _ in j] == [n for n, _ in c], (cname, j, c)
    assert [t for _, t in j] == [t for _, t in c], (cname, j, c)


def header_enums():
    vals = {}
    for name, val in re.findall(r"\b(NQCD_[A-Z0-9_]+)\s*=\s*(-?\d+)", HEADER):
        vals[name] = int(val)
    return vals


def test_julia_constants_match_the_header():
    enums = header_enums()
    found = 0
    for jname, val in re.findall(r"^const ((?:METHOD|MODEL|PREC|INIT|SAMPLE)_\w+) = Int32\((-?\d+)\)", JL, flags=re.M):
        assert enums["NQCD_" + jname] == int(val), jname
        found += 1
    assert found == 6 + 6 + 3 + 4 + 3
    abi = int(re.search(r"#define NQCD_ABI_VERSION (\d+)", HEADER).group(1))
    assert f"const ABI_VERSION = Int32({abi})" in JL


def test_julia_philox_constants_and_streams_match_the_engine():
    for name in ("M0", "M1", "W0", "W1"):
        c = int(re.search(r"\b%s = (0x[0-9A-Fa-f]+)u" % name, MATH).group(1), 16)
        j = int(re.search(r"const PHILOX_%s = (0x[0-9A-Fa-f]+)" % name, JL).group(1), 16)
        assert c == j, name
    streams = dict((n, int(v)) for n, v in re.findall(r"\b(RNG_\w+) = (\d+),", MATH))
    for n, v in re.findall(r"const (RNG_\w+) = UInt32\((\d+)\)", JL):
        assert streams[n] == int(v), n
    assert len(streams) == 6


def test_julia_philox_known_answers_equal_the_oracle():
    table = JL[JL.index("const KNOWN_ANSWERS"):]
    table = table[:table.index("\n)\n")]
    rows = re.findall(r"\(\((.*?)\), \((.*?)\),\s*\((.*?)\)\)", table, flags=re.S)
    assert len(rows) == 3
    for ctr, key, out in rows:
        ctr, key, out = ([int(x, 16) for x in s.split(",")] for s in (ctr, key, out))
        assert O.philox(ctr, key) == out


def test_julia_philox_round_structure():
    """The round body and key schedule read as the engine's: (hi1 ^ c1 ^ k0,
    lo1, hi0 ^ c3 ^ k1, lo0) with hi0/lo0 = M0 * c0, hi1/lo1 = M1 * c2, and the
    words taken in (traj low, traj high, step, stream) / (seed low, seed high)
    order; the 53-bit uniform is the top 53 bits of (w1, w2) times 2^-53."""
    assert "hi0, lo0 = mulhilo(PHILOX_M0, c0)" in JL
    assert "hi1, lo1 = mulhilo(PHILOX_M1, c2)" in JL
    assert "c0, c1, c2, c3 = hi1 ⊻ c1 ⊻ k0, lo1, hi0 ⊻ c3 ⊻ k1, lo0" in JL
    assert "philox4x32_10(traj % UInt32, (traj >> 32) % UInt32, step, stream, seed % UInt32, (seed >> 32) % UInt32)" in JL
    assert "Float64(((UInt64(hi) << 32) | UInt64(lo)) >> 11) * 0x1p-53" in JL
    # the C side, for the record
    assert "c.x = (uint32_t)traj;" in MATH and "c.y = (uint32_t)(traj >> 32);" in MATH
    assert "return (double)(bits >> 11) * 0x1.0p-53;" in MATH


def test_julia_file_reduction_writes_through_the_reference():
    """FileReduction on the Julia side hands per-trajectory Dictionaries to the
    reference's own FileReduction (reductions.jl:57-91), which writes HDF5; the
    outputs it takes are the ones the Python mirror writes to .npz."""
    assert "reduction isa NQCDynamics.Ensembles.FileReduction" in JL
    assert "message, _ = reduction(nothing, batch, 1:trajectories)" in JL
    jl = re.search(r"const FILE_OUTPUTS = \((.*?)\)", JL).group(1)
    names = [x.strip().lstrip(":") for x in jl.split(",")]
    api = (ROOT / "nqcdynamics.jl_gb300" / "nqcd_gb300" / "api.py").read_text()
    body = api[api.index("def _per_trajectory"):api.index("def _metal_config")]
    assert sorted(names) == sorted(set(re.findall(r'"(Output\w+)"', body)))
