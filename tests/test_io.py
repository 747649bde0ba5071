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


def _ref_misc_or_skip():
    from oracle import oracle as O
    if not O.ref_available("misc"):
        pytest.skip("the reference's misc.c was not built here (make -C oracle ref)")
    return O


GRAPH_FILES = {
    # comment lines, a line stopped by its 0, a self pair, lower neighbours dropped
    "details": "% a comment\n% another\n4 4\n2 3\n1 4 0 3\n1 3\n2\n",
    # isolated nodes and extra spaces; neighbours listed in any order
    "spaces": "6 3\n  3   2\n1\n1 6 \n\n\n3\n",
    # no neighbour lines at all for the last nodes (counted as empty)
    "short": "5 1\n2\n1\n",
}


@pytest.mark.parametrize("name", sorted(GRAPH_FILES))
def test_read_graph_matches_reference_reader(built_lib, tmp_path, name, capfd):
    """irr_read_graph against moldyn's own ReadInputGraph compiled from misc.c:
    the same pairs in the same order.  That build defines CSTYLE, so its pairs
    are 0-based, which is irr_read_graph's default (one_based = 0)."""
    O = _ref_misc_or_skip()
    import irregular_gb300 as irr
    path = tmp_path / f"{name}.mesh"
    path.write_text(GRAPH_FILES[name])
    ours = irr.read_graph(str(path))
    ref, n = O.ref_read_graph(str(path), ours.shape[0] + 8)
    capfd.readouterr()  # the reference prints its header line
    assert n == int(GRAPH_FILES[name].split("\n")[[i for i, l in enumerate(
        GRAPH_FILES[name].split("\n")) if not l.startswith("%")][0]].split()[0])
    assert np.array_equal(ours, ref)


def test_read_graph_matches_reference_reader_on_a_written_list(built_lib, tmp_path, capfd):
    """A 2,048-node random moldyn half list written in the adjacency format and
    read back by both readers."""
    O = _ref_misc_or_skip()
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    path = str(tmp_path / "g.mesh")
    irr.write_graph(path, c["pos"].shape[0], c["edges"])
    ours = irr.read_graph(path)
    ref, n = O.ref_read_graph(path, ours.shape[0] + 8)
    capfd.readouterr()
    assert n == c["pos"].shape[0]
    assert np.array_equal(ours, ref)
    assert np.array_equal(irr.read_graph(path, one_based=True), ref + 1)


def test_read_coords_matches_reference_reader(built_lib, tmp_path):
    O = _ref_misc_or_skip()
    import irregular_gb300 as irr
    rng = np.random.default_rng(5)
    xyz = rng.random((777, 3)) * 108.045548
    path = str(tmp_path / "c.xyz")
    irr.write_coords(path, xyz)
    # a hand-formatted file too: mixed separators and exponents
    path2 = tmp_path / "h.xyz"
    path2.write_text("1 2 3\n4.5e-1\t-6 2\n7.25 1e3 -0.0\n")
    for p, n in ((path, 777), (str(path2), 3)):
        assert np.array_equal(irr.read_coords(p, n), O.ref_read_coords(p, n))
