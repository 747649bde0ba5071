"""The drivers' graph and coordinate file formats (host code, CPU)."""
import numpy as np
import pytest

from helpers import load_golden


def test_graph_round_trip_of_a_sorted_half_list(built_lib, tmp_path):
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    path = str(tmp_path / "g.mesh")
    irr.write_graph(path, c["pos"].shape[0], c["edges"])
    e = irr.read_graph(path)
    assert np.array_equal(e, c["edges"])
    e1 = irr.read_graph(path, one_based=True)
    assert np.array_equal(e1, c["edges"] + 1)


def test_graph_format_details(built_lib, tmp_path):
    import irregular_gb300 as irr
    path = tmp_path / "small.mesh"
    # comment lines, then 4 nodes / 4 pairs; line 2 stops at the 0; a
    # self-pair (3,3) counts once; neighbours below the node id are not kept
    path.write_text("% a comment\n% another\n4 4\n2 3\n1 4 0 3\n1 3\n2\n")
    e = irr.read_graph(str(path))
    assert e.tolist() == [[0, 1], [0, 2], [1, 3], [2, 2]]


def test_graph_edge_count_mismatch_is_an_error(built_lib, tmp_path):
    import irregular_gb300 as irr
    path = tmp_path / "bad.mesh"
    path.write_text("3 5\n2\n1 3\n2\n")
    with pytest.raises(irr.IrregularError) as ei:
        irr.read_graph(str(path))
    assert ei.value.status == irr.IRR_ERR_STATE


def test_coords_round_trip_exact(built_lib, tmp_path):
    import irregular_gb300 as irr
    rng = np.random.default_rng(3)
    xyz = rng.random((500, 3)) * 108.045548
    path = str(tmp_path / "c.xyz")
    irr.write_coords(path, xyz)
    assert np.array_equal(irr.read_coords(path, 500), xyz)
    with pytest.raises(irr.IrregularError):
        irr.read_coords(path, 499)
