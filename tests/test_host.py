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
