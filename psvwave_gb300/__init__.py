"""psvwave_gb300 -- GB300 (sm_103a) implementation of psvWave's P-SV
finite-difference solver, behind the reference's `fdModel` API.

    import psvwave_gb300 as psvWave
    model = psvWave.fdModel("configuration.ini")
    model.forward_simulate(0)
    ux, uz = model.get_synthetic_data()
"""
from .config import from_dictionary, get_dictionary, to_parameters, write_dictionary
from .batch import Batch
from .model import fdModel

__all__ = ["fdModel", "Batch", "get_dictionary", "write_dictionary", "from_dictionary", "to_parameters"]
__version__ = "0.1.0"
