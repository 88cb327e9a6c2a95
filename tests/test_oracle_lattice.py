"""Lattice index maps of the oracle against the reference's known answers
(src/lattice/test_lattice.hh:35-241, lattices 6 / 4x5 / 4x5x6 cells)."""
import oracle as O


def test_lattice_1d():
    lat = O.Lattice(6)
    assert lat.cellidx_linear2euclidean(5) == (5,)
    assert lat.cellidx_euclidean2linear((3,)) == 3
    assert lat.vertexidx_linear2euclidean(4) == (5,)
    assert lat.vertexidx_euclidean2linear((3,)) == 2
    assert lat.shift_vertexidx(3, (1,)) == 4
    assert lat.shift_vertexidx(3, (-1,)) == 2
    assert lat.shift_vertexidx(4, (-1,)) == 3
    assert lat.fine_vertex_idx(3) == 7
    assert lat.fine_vertex_idx(0) == 1
    assert lat.fine_vertex_idx(2) == 5


def test_lattice_2d():
    lat = O.Lattice(4, 5)
    assert lat.cellidx_linear2euclidean(6) == (2, 1)
    assert lat.cellidx_euclidean2linear((1, 2)) == 9
    # shift_cellidx(5, .) through the index maps
    c = lat.cellidx_linear2euclidean(5)
    for s, want in (((0, 1), 9), ((0, -1), 1), ((1, 0), 6), ((-1, 0), 4)):
        assert lat.cellidx_euclidean2linear((c[0] + s[0], c[1] + s[1])) == want
    assert lat.vertexidx_linear2euclidean(5) == (3, 2)
    assert lat.vertexidx_euclidean2linear((3, 2)) == 5
    assert lat.shift_vertexidx(7, (0, 1)) == 10
    assert lat.shift_vertexidx(7, (0, -1)) == 4
    assert lat.shift_vertexidx(7, (1, 0)) == 8
    assert lat.shift_vertexidx(7, (-1, 0)) == 6
    assert lat.fine_vertex_idx(0) == 8
    assert lat.fine_vertex_idx(7) == 38
    assert lat.fine_vertex_idx(3) == 22


def test_lattice_3d():
    lat = O.Lattice(4, 5, 6)
    assert lat.cellidx_linear2euclidean(53) == (1, 3, 2)
    assert lat.cellidx_euclidean2linear((1, 3, 2)) == 53
    c = lat.cellidx_linear2euclidean(59)
    for s, want in (((0, 1, 0), 63), ((0, -1, 0), 55), ((1, 0, 0), 60), ((-1, 0, 0), 58),
                    ((0, 0, 1), 79), ((0, 0, -1), 39)):
        assert lat.cellidx_euclidean2linear(tuple(c[d] + s[d] for d in range(3))) == want
    assert lat.vertexidx_linear2euclidean(23) == (3, 4, 2)
    assert lat.vertexidx_euclidean2linear((3, 4, 2)) == 23
    for s, want in (((0, 1, 0), 26), ((0, -1, 0), 20), ((1, 0, 0), 24), ((-1, 0, 0), 22),
                    ((0, 0, 1), 35), ((0, 0, -1), 11)):
        assert lat.shift_vertexidx(23, s) == want
    assert lat.fine_vertex_idx(23) == 243


def test_vertex_counts_and_coordinates():
    # Lattice3d(nx, ny, nz) has (nx-1)(ny-1)(nz-1) interior vertices at h*idx
    assert O.Lattice(128, 128, 128).nvertex == 127 ** 3
    assert O.Lattice(256, 256, 256).nvertex == 255 ** 3
    assert O.Lattice(64, 64).nvertex == 63 ** 2
    assert O.Lattice(4, 5, 6).vertex_coordinates(23) == (3 / 4, 4 / 5, 2 / 6)
