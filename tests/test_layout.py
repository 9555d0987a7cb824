"""AoSoA layout, view maps and graph ordering (host logic, no GPU)."""
import numpy as np
import pytest

from pyfr_gb300.backend.types import layout, pack, unpack, view_mapping


@pytest.mark.parametrize('ioshape', [(5, 7), (16, 4, 37), (3, 16, 5, 70),
                                     (4, 4, 32), (2, 1, 1, 1)])
def test_pack_unpack_roundtrip(ioshape):
    nrow, ncol, ld, ds = layout(ioshape, {'align'})
    a = np.random.default_rng(0).normal(size=ioshape)
    flat = pack(a, nrow, ld)
    assert flat.shape == (nrow, ld)
    np.testing.assert_array_equal(unpack(flat, ioshape, ds), a)


def test_aosoa_offsets():
    # element e, variable v of row r sits at r*ld + (e//32)*32*nv + v*32 + e%32
    nupts, nv, ne = 3, 4, 70
    nrow, ncol, ld, ds = layout((nupts, nv, ne), {'align'})
    assert ld == nv*96
    a = np.arange(nupts*nv*ne, dtype=float).reshape(nupts, nv, ne)
    flat = pack(a, nrow, ld).ravel()
    for r, v, e in [(0, 0, 0), (1, 3, 33), (2, 2, 69)]:
        assert flat[r*ld + (e//32)*32*nv + v*32 + e % 32] == a[r, v, e]


def test_view_mapping_formula():
    class M:
        def __init__(self, off, ld):
            self.offset, self.itemsize, self.leaddim = off, 8, ld
    mats = {0: M(0, 320), 1: M(8*1000, 320)}
    m, ld = view_mapping(mats, np.array([0, 1, 1]), np.array([2, 0, 5]),
                         np.array([3, 40, 65]), nvcol=5)
    assert list(m) == [2*320 + 3, 1000 + 0 + 32*5 + 8, 1000 + 5*320 + 64*5 + 1]


def test_graph_topological_order_keeps_deps():
    from pyfr_gb300.backend.types import Graph, Kernel

    class FakeBackend:
        use_cuda_graphs = False
        def fuse(self, k, g):
            return k

    g = Graph(FakeBackend())
    a, b, c, d = (Kernel(name=n) for n in 'abcd')
    g.add(c, deps=[])
    g.add(a)
    g.add(b, deps=[a])
    g.add(d, deps=[b, c])
    g.group([a, b])
    g.commit()
    order = [k.name for k in g.klist]
    assert order.index('a') < order.index('b') < order.index('d')
    assert order.index('c') < order.index('d')
    assert abs(order.index('a') - order.index('b')) == 1
