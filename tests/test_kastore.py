"""Reading .trees files (tskit's kastore container) against files written by
the reference itself (tests/golden/make_trees_files.py) and the columns the
reference reads back from them; malformed files give the reference's errors.
Host code only."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
NAMES = ["sim_n40", "multiallelic_n30", "uncalibrated_n20"]
COLUMNS = ["node_time", "node_flags", "edge_left", "edge_right", "edge_parent", "edge_child",
           "site_position", "site_ancestral_state", "site_ancestral_state_offset",
           "mutation_site", "mutation_node", "mutation_parent", "mutation_derived_state",
           "mutation_derived_state_offset"]


@pytest.mark.parametrize("name", NAMES)
def test_columns_match_reference(name, cuda_lib_cpu):
    from tskit_gb300 import Tables

    t = Tables.load(os.path.join(GOLDEN, name + ".trees"))
    ref = np.load(os.path.join(GOLDEN, name + "_trees.npz"))
    assert t.sequence_length == float(ref["sequence_length"])
    # edges are re-sorted into the statistics' canonical order, which the
    # reference's sorted tables already have
    for c in COLUMNS:
        np.testing.assert_array_equal(getattr(t, c), ref[c], err_msg=c)
    assert t.time_uncalibrated == (ref["time_units"].tobytes() == b"uncalibrated")
    t.check()


def _bytes(name):
    with open(os.path.join(GOLDEN, name + ".trees"), "rb") as f:
        return bytearray(f.read())


def _load_bytes(tmp_path, data):
    from tskit_gb300 import Tables

    p = tmp_path / "x.trees"
    p.write_bytes(bytes(data))
    return Tables.load(str(p))


def test_missing_file(tmp_path, cuda_lib_cpu):
    from tskit_gb300 import LibraryError, Tables
    from tskit_gb300 import _native as nat

    with pytest.raises(LibraryError) as e:
        Tables.load(str(tmp_path / "none.trees"))
    assert e.value.code == nat.ERR_IO


@pytest.mark.parametrize("mutate", ["magic", "truncate", "extend", "size", "name", "version"])
def test_malformed(tmp_path, mutate, cuda_lib_cpu):
    from tskit_gb300 import LibraryError
    from tskit_gb300 import _native as nat

    data = _bytes("sim_n40")
    expect = nat.ERR_FILE_FORMAT
    if mutate == "magic":
        data[1] = ord("X")
    elif mutate == "truncate":
        data = data[: len(data) - 9]
    elif mutate == "extend":
        data += b"\0" * 8
    elif mutate == "size":
        data[16] ^= 1
    elif mutate == "name":
        i = data.find(b"tskit.trees")
        assert i > 0
        data[i + 10] = ord("z")
    elif mutate == "version":
        data[8] = 2  # the container's major version
        expect = nat.ERR_FILE_VERSION_TOO_NEW
    with pytest.raises(LibraryError) as e:
        _load_bytes(tmp_path, data)
    assert e.value.code == expect
