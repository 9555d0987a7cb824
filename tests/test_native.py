"""Native mesh and solution files and the Gmsh importer (CPU).

The records follow the reference's format description
(doc/src/file_format.rst): codec entries, per-element face connectivity
(cidx, off), node valencies, periodic face pairs, the default
partitioning, and the solution's compound records.  Meshes generated here
go through the files and come back with the same interfaces and
boundaries; Gmsh files of structured boxes import to the same meshes; a
hand-written two-element file gives the connectivity worked out by hand
from the format's face numbering."""
import numpy as np
import pytest

from pyfr_gb300.gmsh import GmshReader, fuzzy_lexsort, import_mesh
from pyfr_gb300.inifile import Inifile
from pyfr_gb300.mesh import Mesh, Side, box, mixed_box, periodic_box, tri_box
from pyfr_gb300.native import (NativeFile, NativeFileWriter, corner_nodes,
                               read_mesh, read_soln, read_subset_soln,
                               save_mesh, std_ele, write_soln)
from tests.gmsh_util import box_msh, raise_order


def _pairs(m):
    l, r = m.con
    return {tuple(sorted([a[:3], a[3:]]))
            for a in zip(l.etypes.tolist(), l.eidxs.tolist(),
                         l.fidxs.tolist(), r.etypes.tolist(),
                         r.eidxs.tolist(), r.fidxs.tolist())}


def _bfaces(sd):
    return sorted(zip(sd.etypes.tolist(), sd.eidxs.tolist(),
                      sd.fidxs.tolist()))


def test_container_round_trip(tmp_path):
    dt = np.dtype([('soln', [('rho', float, (3,)), ('E', float, (3,))]),
                   ('aux', [('part-id', np.int64)])])
    a = np.zeros(4, dtype=dt)
    a['soln']['rho'] = np.arange(12).reshape(4, 3)
    w = NativeFileWriter()
    w['grp/sub/data'] = a
    w.set_attr('grp/sub/data', 'pts', np.eye(3))
    w['name'] = 'hello'
    w['version'] = np.int64(2)
    w.save(tmp_path / 'x.pyfrs')
    with NativeFile(tmp_path / 'x.pyfrs') as f:
        assert f['grp/sub/data'].dtype == dt
        assert np.array_equal(f['grp/sub/data'], a)
        assert np.array_equal(f.attrs('grp/sub/data')['pts'], np.eye(3))
        assert f.string('name') == 'hello'
        assert int(f['version']) == 2
        assert f.names() == ['grp', 'name', 'version']
        assert f.names('grp') == ['sub'] and 'grp/sub' in f
        assert 'nothing' not in f


def test_hdf5_needs_h5py(tmp_path):
    p = tmp_path / 'h.pyfrm'
    p.write_bytes(b'\x89HDF\r\n\x1a\n' + bytes(64))
    try:
        import h5py                                       # noqa: F401
        pytest.skip('h5py is installed')
    except ImportError:
        with pytest.raises(RuntimeError, match='h5py'):
            NativeFile(p)


def test_std_ele_corners():
    # Node ordering of the format: x fastest, equi-spaced Lagrange points
    assert np.allclose(std_ele('quad', 2)[:4],
                       [(-1, -1), (0, -1), (1, -1), (-1, 0)])
    assert corner_nodes('quad', 2) == [0, 2, 6, 8]
    assert corner_nodes('tri', 3) == [0, 3, 9]
    assert corner_nodes('hex', 1) == list(range(8))
    assert corner_nodes('pri', 2) == [0, 2, 5, 12, 14, 17]
    assert len(std_ele('tet', 3)) == 20 and corner_nodes('tet', 3)[-1] == 19
    assert len(std_ele('pyr', 2)) == 14
    assert corner_nodes('pyr', 2) == [0, 2, 6, 8, 13]


MESHES = {
    'quad-periodic': lambda: periodic_box('quad', (4, 3), 0.0, 1.0),
    'hex-bounded': lambda: box('hex', (3, 2, 2), 0.0, 1.0,
                               (True, False, True)),
    'hex-pri': lambda: mixed_box(2, -1.0, 1.0, 'hex-pri'),
    'pri-tet': lambda: mixed_box(2, -1.0, 1.0, 'pri-tet'),
    'hex-pyr-tet': lambda: mixed_box(2, -1.0, 1.0, 'hex-pyr-tet'),
    'tri': lambda: tri_box(3, 0.0, 1.0),
}


@pytest.mark.parametrize('name', MESHES)
def test_mesh_round_trip(tmp_path, name):
    m = MESHES[name]()
    fn = tmp_path / 'm.pyfrm'
    uuid = save_mesh(fn, m)
    r = read_mesh(fn)
    assert r.uuid == uuid and r.codec[-1] == 'tag/fluid'
    assert _pairs(r) == _pairs(m)
    for et in m.spts:
        assert np.array_equal(r.spts[et], m.spts[et])
        assert np.array_equal(r.eidxs[et], np.arange(m.spts[et].shape[1]))
    assert set(r.bcon) == set(m.bcon)
    for k in m.bcon:
        assert _bfaces(r.bcon[k]) == _bfaces(m.bcon[k])

    with NativeFile(fn) as f:
        assert int(f['version']) == 2
        nodes = f['nodes']
        nref = sum(len(np.unique(f[f'eles/{et}']['nodes'], axis=None))
                   for et in f.names('eles'))
        assert nodes['valency'].sum() == sum(
            f[f'eles/{et}']['nodes'].size for et in f.names('eles'))
        assert nref >= len(nodes) or len(f.names('eles')) > 1
        # Every face is an interface, a boundary, or a periodic pair member
        npairs = sum(len(f[f'periodic/{k}']) for k in f.names('periodic')) \
            if 'periodic' in f else 0
        assert npairs <= len(m.con[0])
        # Neighbouring elements never share a colour
        for et in f.names('eles'):
            e = f[f'eles/{et}']
            for fi in range(e['faces'].shape[1]):
                c = e['faces']['cidx'][:, fi]
                off = e['faces']['off'][:, fi]
                codec = [x.decode() for x in f['codec']]
                for i in np.flatnonzero(off >= 0):
                    other = codec[c[i]].split('/')[1]
                    assert f[f'eles/{other}']['colour'][off[i]] != \
                        e['colour'][i] or (other == et and off[i] == i)


def test_uuid_depends_on_mesh(tmp_path):
    a = save_mesh(tmp_path / 'a.pyfrm', periodic_box('quad', 3, 0.0, 1.0))
    b = save_mesh(tmp_path / 'b.pyfrm', periodic_box('quad', 3, 0.0, 1.0))
    c = save_mesh(tmp_path / 'c.pyfrm', periodic_box('quad', 3, 0.0, 2.0))
    assert a == b != c


@pytest.mark.parametrize('version', ['2.2', '4.1'])
@pytest.mark.parametrize('n,periodic', [((4, 3), (True, False)),
                                        ((3, 2, 2), (True, False, True)),
                                        ((2, 2, 2), (True, True, True)),
                                        ((2, 3), (False, False))])
def test_gmsh_box(tmp_path, version, n, periodic):
    fn = tmp_path / 'g.pyfrm'
    import_mesh(box_msh(n, periodic, version), fn)
    m = read_mesh(fn)
    et = 'quad' if len(n) == 2 else 'hex'
    ref = box(et, n, 0.0, 1.0, periodic)
    assert _pairs(m) == _pairs(ref)
    assert np.allclose(m.spts[et], ref.spts[et])
    assert set(m.bcon) == set(ref.bcon)
    for k in ref.bcon:
        assert _bfaces(m.bcon[k]) == _bfaces(ref.bcon[k])
    with NativeFile(fn) as f:
        per = f.names('periodic') if 'periodic' in f else []
        assert sorted(per) == [str(d) for d in range(len(n)) if periodic[d]]


# Two unit quads side by side on [0, 2] x [0, 1]; nodes 1..6 numbered x
# fastest; Gmsh lists quad vertices around the element
TWO_QUADS = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
4
1 10 "Wall"
1 11 "inlet"
1 12 "outlet"
2 20 "fluid"
$EndPhysicalNames
$Nodes
6
1 0 0 0
2 1 0 0
3 2 0 0
4 0 1 0
5 1 1 0
6 2 1 0
$EndNodes
$Elements
8
1 1 2 10 1 1 2
2 1 2 10 1 2 3
3 1 2 10 1 4 5
4 1 2 10 1 5 6
5 1 2 11 2 1 4
6 1 2 12 3 3 6
7 3 2 20 4 1 2 5 4
8 3 2 20 4 2 3 6 5
$EndElements
"""


def test_gmsh_two_quads(tmp_path):
    """Quad faces are numbered 0 (y = -1), 1 (x = +1), 2 (y = +1),
    3 (x = -1); element 0's face 1 meets element 1's face 3."""
    nodes, eles, codec, pmap = GmshReader(TWO_QUADS).records()
    assert codec == ['eles/quad', 'eles/quad/face/0', 'eles/quad/face/1',
                     'eles/quad/face/2', 'eles/quad/face/3', 'bc/wall',
                     'bc/inlet', 'bc/outlet', 'tag/fluid']
    q = eles['quad']
    assert q['nodes'].tolist() == [[0, 1, 3, 4], [1, 2, 4, 5]]
    wall, inlet, outlet = 5, 6, 7
    assert q['faces'].tolist() == [
        [(wall, -1), (4, 1), (wall, -1), (inlet, -1)],
        [(wall, -1), (outlet, -1), (wall, -1), (2, 0)]]
    assert q['tags'].tolist() == [1, 1] and pmap == {}

    import_mesh(TWO_QUADS, tmp_path / 'q.pyfrm')
    with NativeFile(tmp_path / 'q.pyfrm') as f:
        assert f['nodes']['valency'].tolist() == [1, 2, 1, 1, 2, 1]
        assert np.array_equal(f['nodes']['location'][4], [1.0, 1.0])
        assert f['eles/quad']['colour'].tolist() == [0, 1]
        regions = f.attrs('partitionings/1/eles')['regions']
        assert regions.tolist() == [[0, 2]]
    m = read_mesh(tmp_path / 'q.pyfrm')
    assert _pairs(m) == {(('quad', 0, 1), ('quad', 1, 3))}
    assert _bfaces(m.bcon['wall']) == [('quad', 0, 0), ('quad', 0, 2),
                                       ('quad', 1, 0), ('quad', 1, 2)]


@pytest.mark.parametrize('bad,msg', [
    ('"inlet"\n1 12 "outlet"', 'Duplicate physical name'),
    ('"outlet"', None),
])
def test_gmsh_errors(bad, msg):
    if msg:
        txt = TWO_QUADS.replace('"outlet"', bad.split('\n')[0])
        with pytest.raises(ValueError, match=msg):
            GmshReader(txt)
    # A boundary element dropped leaves a face unpaired
    lines = TWO_QUADS.splitlines()
    i = lines.index('6 1 2 12 3 3 6')
    txt = '\n'.join(lines[:i] + lines[i + 1:]).replace('\n8\n1 1', '\n7\n1 1')
    with pytest.raises(ValueError, match='Unpaired'):
        GmshReader(txt + '\n').records()
    # A second-order type with a first-order node list is refused
    txt = TWO_QUADS.replace('7 3 2 20 4 1 2 5 4', '7 10 2 20 4 1 2 5 4')
    with pytest.raises(ValueError, match='node count'):
        GmshReader(txt)
    # One side of a periodic pair alone
    txt = TWO_QUADS.replace('"inlet"', '"periodic_0_l"')
    with pytest.raises(ValueError, match='Unpaired periodic'):
        GmshReader(txt)


def test_fuzzy_lexsort():
    pts = np.array([[0.0, 1e-9, 1.0, 0.0], [2.0, 1.0, 0.0, 0.5]])
    # Columns 0, 1 and 3 tie in x (within 1e-6) and are ordered by y
    assert fuzzy_lexsort(pts, range(4)) == [3, 1, 0, 2]


def _soln_mesh():
    m = periodic_box('quad', (3, 2), 0.0, 1.0)
    m.uuid = 'abc'
    # File numbers of the local elements: a permutation
    m.eidxs = {'quad': np.array([4, 0, 5, 1, 3, 2])}
    return m


def test_soln_round_trip(tmp_path):
    m = _soln_mesh()
    rng = np.random.default_rng(3)
    u = rng.standard_normal((16, 4, 6))
    cfg = Inifile()
    cfg.set('solver', 'order', 3)
    stats = Inifile()
    stats.set('solver-time-integrator', 'tcurr', '0.25')
    fields = ['rho', 'rhou', 'rhov', 'E']
    upts = {'quad': rng.random((16, 2))}
    fn = tmp_path / 's.pyfrs'
    write_soln(fn, m, {'quad': u}, upts, fields, cfg, stats,
               prevcfgs={'config-0': '[solver]\norder = 2\n'},
               state={'intg/ctrl': np.array([1e-3, 0.5])})
    s = read_soln(fn, m)
    assert s.fields == fields
    assert np.array_equal(s.data['quad'], u)
    assert s.stats.getfloat('solver-time-integrator', 'tcurr') == 0.25
    assert s.stats.get('data', 'prefix') == 'soln'
    assert sorted(s.prevcfgs) == ['config-0', 'config-1']
    assert s.config.getint('solver', 'order') == 3
    assert np.array_equal(s.state['intg/ctrl'], [1e-3, 0.5])
    assert s.aux['quad']['part-id'].tolist() == [0]*6

    with NativeFile(fn) as f:
        rec = f['soln/p3-quad']
        # Stored at the elements' file numbers, one record per element
        assert np.array_equal(rec['soln']['rhou'][4], u[:, 1, 0])
        assert np.array_equal(f.attrs('soln/p3-quad')['pts'], upts['quad'])
        assert f.string('mesh-uuid') == 'abc'

    m2 = _soln_mesh()
    m2.uuid = 'other'
    with pytest.raises(RuntimeError, match='Invalid solution'):
        read_soln(fn, m2)


def test_config_chain(tmp_path):
    """The configuration history grows only when the configuration
    changes (pyfr/integrators/base.py:369-381)."""
    m = _soln_mesh()
    cfg = Inifile()
    cfg.set('solver', 'order', 1)
    u = {'quad': np.zeros((4, 4, 6))}
    up = {'quad': np.zeros((4, 2))}
    write_soln(tmp_path / 'a.pyfrs', m, u, up, list('abcd'), cfg, None,
               prevcfgs={'config-0': cfg.tostr()})
    s = read_soln(tmp_path / 'a.pyfrs', m)
    assert sorted(s.prevcfgs) == ['config-0']


def test_restart_records_without_gpu(tmp_path):
    """A Side-built mesh keeps boundary names through the file."""
    spts = periodic_box('quad', 2, 0.0, 1.0).spts
    lhs = Side(['quad']*2, [0, 1], [1, 1])
    rhs = Side(['quad']*2, [1, 0], [3, 3])
    bcon = {'lo': Side(['quad']*2, [0, 1], [0, 0]),
            'hi': Side(['quad']*2, [0, 1], [2, 2])}
    spts = {'quad': spts['quad'][:, :2]}
    m = Mesh(ndims=2, spts=spts, con=(lhs, rhs), bcon=bcon)
    save_mesh(tmp_path / 'm.pyfrm', m)
    r = read_mesh(tmp_path / 'm.pyfrm')
    assert set(r.bcon) == {'lo', 'hi'}
    assert len(r.con[0]) == 2


def test_soln_gradients_round_trip(tmp_path):
    m = _soln_mesh()
    rng = np.random.default_rng(4)
    u = rng.standard_normal((16, 4, 6))
    g = rng.standard_normal((2, 16, 4, 6))
    cfg = Inifile()
    cfg.set('solver', 'order', 3)
    write_soln(tmp_path / 'g.pyfrs', m, {'quad': u}, {'quad': np.zeros((16, 2))},
               ['rho', 'rhou', 'rhov', 'E'], cfg, None, grads={'quad': g})
    s = read_soln(tmp_path / 'g.pyfrs', m)
    assert np.array_equal(s.grad_data['quad'], g)
    with NativeFile(tmp_path / 'g.pyfrs') as f:
        rec = f['soln/p3-quad']
        # grad.rhou of the element stored first (file number 0 = local 1)
        assert np.array_equal(rec['grad']['rhou'][0], g[:, :, 1, 1])


# The two quads as second-order elements: 9-node quadrilaterals and 3-node
# lines (vertices first, then edge midpoints, then the centre, as Gmsh
# lists them); nodes 7-13 are the extra nodes
TWO_QUADS_P2 = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
4
1 10 "Wall"
1 11 "inlet"
1 12 "outlet"
2 20 "fluid"
$EndPhysicalNames
$Nodes
13
1 0 0 0
2 1 0 0
3 2 0 0
4 0 1 0
5 1 1 0
6 2 1 0
7 0.5 0 0
8 1.5 0 0
9 0.5 1 0
10 1.5 1 0
11 0 0.5 0
12 1 0.5 0
13 2 0.5 0
14 0.5 0.5 0
15 1.5 0.5 0
$EndNodes
$Elements
8
1 8 2 10 1 1 2 7
2 8 2 10 1 2 3 8
3 8 2 10 1 4 5 9
4 8 2 10 1 5 6 10
5 8 2 11 2 1 4 11
6 8 2 12 3 3 6 13
7 10 2 20 4 1 2 5 4 7 12 9 11 14
8 10 2 20 4 2 3 6 5 8 13 10 12 15
$EndElements
"""


def test_gmsh_straight_high_order(tmp_path):
    """Straight second-order elements read as their vertices, giving the
    connectivity of the first-order file; a curved one raises."""
    txt = TWO_QUADS_P2.replace('\n13\n1 0 0 0', '\n15\n1 0 0 0')
    nodes, eles, codec, pmap = GmshReader(txt).records()
    _, eles1, codec1, _ = GmshReader(TWO_QUADS).records()
    assert codec == codec1
    assert eles['quad']['faces'].tolist() == eles1['quad']['faces'].tolist()
    assert eles['quad']['nodes'].tolist() == eles1['quad']['nodes'].tolist()
    import_mesh(txt, tmp_path / 'p2.pyfrm')
    assert _pairs(read_mesh(tmp_path / 'p2.pyfrm')) == \
        {(('quad', 0, 1), ('quad', 1, 3))}

    curved = txt.replace('\n14 0.5 0.5 0\n', '\n14 0.55 0.5 0\n')
    with pytest.raises(ValueError, match='Curved'):
        GmshReader(curved)


@pytest.mark.parametrize('order', [2, 3, 4])
def test_gmsh_straight_high_order_hexes(order):
    """Straight hexahedra (and their quadrilateral boundary faces) of
    orders 2-4 read as the first-order mesh; a node moved off the lattice
    raises, also when it moves out of a boundary face's plane in z."""
    lin = box_msh((2, 2, 2), (True, False, False))
    _, eles1, codec1, _ = GmshReader(lin).records()
    _, eles, codec, _ = GmshReader(raise_order(lin, order)).records()
    assert codec == codec1
    for k in ('nodes', 'faces'):
        assert eles['hex'][k].tolist() == eles1['hex'][k].tolist()

    # An interior lattice node of the first hexahedron, moved in x
    first_hex = 1 + sum(1 for ln in lin.split('\n') if ' 3 2 ' in ln[:12])
    with pytest.raises(ValueError, match='Curved'):
        GmshReader(raise_order(lin, order, (first_hex, 0, (0.02, 0, 0))))
    # A boundary quadrilateral (the first facet, on y = lo) bent in z
    with pytest.raises(ValueError, match='Curved'):
        GmshReader(raise_order(lin, order, (1, 0, (0, 0, 0.02))))


def test_gmsh_high_order_import_memory():
    """The straightness check of high-order elements works in bounded
    chunks: importing 3072 order-3 hexahedra stays far below the
    (elements x nodes x lattice points) distance table of one pass (about
    three times that table when done at once)."""
    import tracemalloc
    txt = raise_order(box_msh((16, 16, 12), (True, True, True)), 3)
    tracemalloc.start()
    GmshReader(txt)
    _, peak = tracemalloc.get_traced_memory()
    tracemalloc.stop()
    one_pass = 3072*64*64*3*8
    assert peak < one_pass, peak


def test_subset_solution(tmp_path):
    """A solution of some elements only: records in ascending element
    number with a -idxs array; read back as a cut-down mesh, refused for a
    restart (pyfr/writers/native.py:237-245, pyfr/readers/native.py:
    113-271)."""
    m = _soln_mesh()
    u = np.random.default_rng(5).standard_normal((16, 4, 6))
    cfg = Inifile()
    cfg.set('solver', 'order', 3)
    sel = np.array([3, 0, 5])               # local elements; numbers 1, 4, 2
    write_soln(tmp_path / 's.pyfrs', m, {'quad': u}, {'quad': np.zeros((16, 2))},
               ['rho', 'rhou', 'rhov', 'E'], cfg, None,
               subset={'quad': sel})
    with NativeFile(tmp_path / 's.pyfrs') as f:
        assert f['soln/p3-quad-idxs'].tolist() == [1, 2, 4]
        assert len(f['soln/p3-quad']) == 3
    with pytest.raises(RuntimeError, match='Subset'):
        read_soln(tmp_path / 's.pyfrs', m)
    sub, s = read_subset_soln(tmp_path / 's.pyfrs', m)
    assert sub.eidxs['quad'].tolist() == [1, 2, 4]
    loc = [3, 5, 0]
    assert np.array_equal(s.data['quad'], u[:, :, loc])
    assert np.array_equal(sub.spts['quad'], m.spts['quad'][:, loc])
    assert sub.con is None

    # Curved flags follow their elements
    from dataclasses import replace
    mc = replace(m, spts_curved={'quad': np.array([0, 1, 0, 1, 0, 0], bool)})
    subc, _ = read_subset_soln(tmp_path / 's.pyfrs', mc)
    assert subc.spts_curved['quad'].tolist() == [True, False, False]

    # A file element number that the mesh lacks is an error
    mcut = replace(m, spts={'quad': m.spts['quad'][:, :4]},
                   eidxs={'quad': m.eidxs['quad'][:4]} if m.eidxs else None)
    with pytest.raises(ValueError, match='not in the mesh'):
        read_subset_soln(tmp_path / 's.pyfrs', mcut)
