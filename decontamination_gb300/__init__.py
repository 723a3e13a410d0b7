"""GB300-native batch self-organising maps: a drop-in for the SOM_Batch hot path of lpsc-euclid/decontamination.

``SOM_Batch`` / ``SOM_Abstract`` mirror the reference classes
(decontamination/algo/som_batch.py, decontamination/algo/som_abstract.py); their
compute runs in libsomgb.so (hand-written sm_103a CUDA kernels behind a C ABI,
include/somgb.h). There is no CPU fallback. Around them: ``SOM_PCA`` and
``Covariance`` (the PCA initialisation, algo/som_pca.py, algo/covariance.py) and
``HypParamFinder_SOM`` (the map-size / radius grid search,
algo/hyparam_finder_som.py), and the request loop in ``serve``.
"""

from .som_abstract import SOM_Abstract
from .som_batch import SOM_Batch, asymptotic_decay
from .covariance import Covariance
from .som_pca import SOM_PCA
from .hyparam_finder_som import HypParamFinder_SOM
from ._dataset import dataset_to_generator_builder

__all__ = ['SOM_Abstract', 'SOM_Batch', 'SOM_PCA', 'Covariance', 'HypParamFinder_SOM', 'asymptotic_decay',
           'dataset_to_generator_builder']
