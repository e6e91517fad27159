"""The voxeliser's float stand-ins against the double arithmetic they
replace, compiled for the host from the same headers the device uses.

The float frame (csrc/frame_rows.cuh) against the double formula it
replaces (mat3.js:71-87, each entry rounded to float32 as the
reference's Float32Array stores it): the header is compiled for the host
with contraction off -- its operations are single IEEE float operations
and fmaf, the same on the device -- and every entry it certifies must equal
the double path's bit for bit, signed zeros included, over random unit and
non-unit quaternions and special values. Unit quaternions must nearly all
be certified (the rest fall back to double on the device).
"""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    compiler = shutil.which("g++")
    if compiler is None:
        pytest.skip("no g++")
    out = tmp_path_factory.mktemp("frame_rows") / "check"
    subprocess.run([compiler, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                    f"-I{ROOT / 'visionary-sim_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "float_checks" / "check_frame_rows.cpp"), "-o", str(out)], check=True)
    return out


def test_float_frame_equals_double_path(harness):
    run = subprocess.run([str(harness), "3000000"], capture_output=True, text=True)
    assert run.returncode == 0, run.stdout + run.stderr
    m = re.search(r"cases (\d+) certified (\d+) .* mismatches (\d+)", run.stdout)
    assert m and int(m.group(3)) == 0
    # a mix with out-of-range specials: most, not all, are certified
    assert int(m.group(2)) > 0.8 * int(m.group(1))


@pytest.fixture(scope="module")
def bounds_harness(tmp_path_factory):
    compiler = shutil.which("g++")
    if compiler is None:
        pytest.skip("no g++")
    out = tmp_path_factory.mktemp("float_bounds") / "check"
    subprocess.run([compiler, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                    f"-I{ROOT / 'visionary-sim_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "float_checks" / "check_float_bounds.cpp"), "-o", str(out)], check=True)
    return out


def test_reach_bracket_float_cells_and_samples(bounds_harness):
    """csrc/float_bounds.cuh: V8's hypot of the double products lies inside
    the float reach estimate's bracket (and its float-rounded bounds); every
    box-edge cell the float test decides is the double division's,
    positions within a few ulps of a cell boundary included; and every
    sample the float sample test decides is decided the same by the double
    evaluation, surfaces within a few ulps of a sample included."""
    run = subprocess.run([str(bounds_harness), "1500000"], capture_output=True, text=True)
    assert run.returncode == 0, run.stdout + run.stderr
    m = re.search(r"reach checked (\d+) bad (\d+); cells tried (\d+) decided (\d+) bad (\d+); "
                  r"samples (\d+) decided (\d+) bad (\d+)", run.stdout)
    assert m and int(m.group(2)) == 0 and int(m.group(5)) == 0 and int(m.group(8)) == 0
    assert int(m.group(4)) > 0.6 * int(m.group(3))
    assert int(m.group(7)) > 0.9 * int(m.group(6))
