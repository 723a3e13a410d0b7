"""Host-side logic of the drop-in that needs no GPU: construction, topography, initialisation, sigma schedule,
dataset protocol and argument errors (they are raised before any device work)."""

import numpy as np
import pytest

import decontamination_gb300 as dg
from decontamination_gb300 import _dataset


def test_constructor_defaults():
    som = dg.SOM_Batch(6, 10, 3)
    assert som.topology == 'hexagonal' and som.dtype == np.float32
    assert som.sigma == 5.0 and som.m == 6 and som.n == 10 and som.dim == 3
    assert som.weights.shape == (60, 3) and som.centroids.shape == (6, 10, 3)
    assert som._header_extra == {'mode': '__MODE__', 'sigma': '_sigma', 'n_epochs': '_n_epochs',
                                 'n_vectors': '_n_vectors'}


@pytest.mark.parametrize('topology', ['square', 'hexagonal'])
def test_topography_matches_oracle(oracle, topology):
    som = dg.SOM_Batch(7, 5, 2, topology=topology)
    assert np.array_equal(som._topography, oracle.topography(7, 5, topology))
    assert som._topography.dtype == np.float32


def test_init_rand_is_numpy_stream():
    som = dg.SOM_Batch(4, 4, 4)
    som.init_rand(seed=0)
    assert np.array_equal(som.weights, np.random.default_rng(0).random((16, 4), dtype=np.float32))


def test_init_from_checks_compatibility():
    a = dg.SOM_Batch(3, 3, 2, topology='square')
    a.init_rand(1)
    b = dg.SOM_Batch(3, 3, 2, topology='square')
    b.init_from(a)
    assert np.array_equal(a.weights, b.weights)
    with pytest.raises(TypeError):
        dg.SOM_Batch(3, 3, 2, topology='hexagonal').init_from(a)
    with pytest.raises(TypeError):
        dg.SOM_Batch(3, 3, 2, dtype=np.float64, topology='square').init_from(a)


def test_invalid_training_method():
    som = dg.SOM_Batch(2, 2, 2)
    with pytest.raises(ValueError):
        som.train(np.zeros((4, 2), np.float32))
    with pytest.raises(ValueError):
        som.train(np.zeros((4, 2), np.float32), n_epochs=1, n_vectors=3)


def test_asymptotic_decay_schedule(oracle):
    for e, E in [(0, 10), (3, 10), (9, 10), (19, 20)]:
        assert dg.asymptotic_decay(e, E) == oracle.decay(e, E)


def test_dataset_protocol_and_alignment():
    x = np.zeros((5, 2), np.float32)
    b = dg.dataset_to_generator_builder(x)
    assert list(b()())[0] is x
    assert dg.dataset_to_generator_builder(None) is None
    chunks = [np.zeros((3, 2)), np.zeros((2, 2))]
    builder = lambda: lambda: iter(chunks)
    assert dg.dataset_to_generator_builder(builder) is builder
    bad_w = lambda: lambda: iter([np.zeros(2), np.zeros(3)])
    with pytest.raises(ValueError, match='aligned'):
        list(_dataset.iterate_chunks(builder, bad_w, np.float32, device=None))


def test_hdf5_round_trip(tmp_path):
    pytest.importorskip('h5py')
    som = dg.SOM_Batch(3, 4, 2, topology='square', sigma=1.5)
    som.init_rand(2)
    path = str(tmp_path / 'som.h5')
    som.save(path)
    other = dg.SOM_Batch(1, 1, 1)
    other.load(path)
    assert other.m == 3 and other.n == 4 and other.sigma == 1.5 and other.topology == 'square'
    assert np.array_equal(other.weights, som.weights)


class _FakeH5:
    """A stand-in for the h5py module (absent here): File objects over an in-memory store that records groups,
    attributes and datasets the way h5py returns them (numbers as numpy scalars, arrays as arrays)."""

    files = {}

    class Group(dict):
        def __init__(self):
            super().__init__()
            self.attrs = _FakeH5.Attrs()

        def create_group(self, name, track_order=None):
            g = _FakeH5.Group()
            self[name] = g
            return g

        def create_dataset(self, name, data, shape, dtype):
            arr = np.array(data, dtype=dtype).reshape(shape)
            self[name] = arr
            return arr

    class Attrs(dict):
        def __setitem__(self, k, v):
            if isinstance(v, bool):
                v = np.bool_(v)
            elif isinstance(v, (int, np.integer)):
                v = np.int64(v)
            elif isinstance(v, (float, np.floating)):
                v = np.float64(v)
            super().__setitem__(k, v)

    class File:
        def __init__(self, filename, mode='r'):
            if mode == 'w':
                _FakeH5.files[filename] = _FakeH5.Group()
            self.root = _FakeH5.files[filename]

        def __enter__(self):
            return self.root

        def __exit__(self, *exc):
            return False


@pytest.fixture
def fake_h5py(monkeypatch):
    import sys
    import types
    mod = types.ModuleType('h5py')
    mod.File = _FakeH5.File
    monkeypatch.setitem(sys.modules, 'h5py', mod)
    _FakeH5.files.clear()
    return _FakeH5


def test_hdf5_layout_and_round_trip_without_h5py(fake_h5py):
    """The reference's HDF5 layout (algo/som_abstract.py:188-319, algo/som_batch.py:75-81, algo/som_pca.py:78-84):
    one group 'model' whose attributes are the header fields and whose datasets are the weights and error
    histories; saving and loading gives the same model back."""
    som = dg.SOM_Batch(3, 4, 2, topology='square', sigma=1.5)
    som.init_rand(2)
    som._n_epochs = 7
    som._quantization_errors = np.array([0.5, 0.25])
    som._topographic_errors = np.array([0.1, 0.05])
    som.save('som.h5')
    g = fake_h5py.files['som.h5']['model']
    assert set(g.attrs) == {'mode', 'sigma', 'n_epochs', 'n_vectors', 'm', 'n', 'dim', 'topology'}
    assert set(g) == {'weights', 'quantization_errors', 'topographic_errors'}
    assert g.attrs['mode'] == 'batch' and g.attrs['topology'] == 'square' and g.attrs['m'] == 3
    assert g['weights'].dtype == np.float32 and g['weights'].shape == som._weights.shape
    other = dg.SOM_Batch(1, 1, 1)
    other.load('som.h5')
    assert (other.m, other.n, other.dim, other.topology, other.sigma) == (3, 4, 2, 'square', 1.5)
    assert other._n_epochs == 7 and other._n_vectors == 0
    assert np.array_equal(other.weights, som.weights)
    # every dataset comes back in the map's dtype, as the reference casts it (algo/som_abstract.py:307-309)
    assert other.quantization_errors.dtype == np.float32
    assert np.array_equal(other.quantization_errors, som.quantization_errors.astype(np.float32))
    assert np.array_equal(other.topographic_errors, som.topographic_errors.astype(np.float32))
    assert other._topography.shape == (12, 2)          # rebuilt for the loaded grid

    pca = dg.SOM_PCA(4, 5, 3, topology='hexagonal')
    pca.init_rand(3)
    pca.save('pca.h5')
    g = fake_h5py.files['pca.h5']['model']
    assert set(g.attrs) == {'mode', 'scale_by_variance', 'apply_cdf', 'cdf_gain', 'm', 'n', 'dim', 'topology'}
    assert g.attrs['mode'] == 'pca'
    back = dg.SOM_PCA(1, 1, 2)
    back.load('pca.h5')
    assert (back.m, back.n, back.dim, back.topology) == (4, 5, 3, 'hexagonal')
    assert np.array_equal(back.weights, pca.weights)


@pytest.mark.parametrize('n', [2 * _dataset.PIECE_ROWS, 2 * _dataset.PIECE_ROWS + 7, 3 * _dataset.PIECE_ROWS - 1,
                               12_582_912, 12_582_912 + 13, 50_331_648, 7 * _dataset.PIECE_ROWS + 1])
def test_piece_edges_cover_the_chunk(n):
    """Host chunks are copied in 2 .. MAX_PIECES pieces whose interior edges are multiples of 16 rows (16-byte aligned
    rows for any D), covering every row once."""
    e = _dataset.piece_edges(n)
    k = len(e) - 1
    assert 2 <= k <= _dataset.MAX_PIECES
    assert k == max(2, min(_dataset.MAX_PIECES, n // _dataset.PIECE_ROWS))
    assert e[0] == 0 and e[-1] == n
    assert all(a <= b for a, b in zip(e, e[1:]))
    assert all(v % 16 == 0 for v in e[:-1])
    sizes = [b - a for a, b in zip(e, e[1:])]
    assert max(sizes) - min(sizes) <= 32


def test_regrouping_is_decided_without_a_device():
    """Rows are regrouped between epochs only for the tensor-core form on maps of more than one 256-unit column tile,
    catalogues of 1024 rows or more, and (under auto) passes of at least 2^22 sample-units; these cases are decided
    before any device query."""
    import decontamination_gb300 as dg
    small = dg.SOM_Batch(8, 8, 16)
    assert not small._regroups(10_000_000)            # one column tile
    som = dg.SOM_Batch(32, 32, 16)
    assert not som._regroups(512)                     # too few rows
    som.bmu_algo = 'fp32'
    assert not som._regroups(10_000_000)              # the CUDA-core form
    som.bmu_algo = 'auto'
    assert not som._regroups(2_000)                   # auto takes the CUDA-core form below 2^22 sample-units
