"""Galaxy-number-density maps from a trained map, in one pass over the footprint.

``Decontamination_SOM`` (decontamination/decontamination_som.py:542-669, a pipeline class outside this package)
computes its footprint winners after training and then two activation maps of the same footprint (weighted by the
corrected galaxy number density, and unweighted) before forming the density per unit and per pixel. ``compute_gndm``
gives the same quantities from ``SOM_Abstract.get_footprint_maps``: one BMU pass and one histogram kernel instead of
three BMU passes. The arithmetic after the maps is the reference's ``_compute_gndm`` (decontamination_som.py:603-626).
"""

import typing

import numpy as np

__all__ = ['compute_gndm']


def compute_gndm(som, footprint_systematics, corrected_galaxy_number_density) -> typing.Dict[str, np.ndarray]:
    """Returns catalog_activation_map, footprint_activation_map, winners, n_gal, n_pix, gnd and gndm."""
    cat, foot, winners = som.get_footprint_maps(footprint_systematics, corrected_galaxy_number_density)
    n_gal = np.sum(cat)
    n_pix = np.sum(foot)
    gnd = np.divide(cat, foot, out=np.full(cat.shape, np.nan, dtype=som.dtype), where=foot > 0.0)
    gndm = gnd.reshape(som.m * som.n)[winners]
    return dict(catalog_activation_map=cat, footprint_activation_map=foot, winners=winners, n_gal=n_gal,
                n_pix=n_pix, gnd=gnd, gndm=gndm)
