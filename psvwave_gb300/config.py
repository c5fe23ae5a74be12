"""Configuration dictionaries and INI files in the reference's format
(psvWave/__init__.py:34-125, src/fdModel.cpp:470-523)."""
import configparser
import copy


_DEFAULTS = {
    "domain": {"nt": 2000, "nx_inner": 400, "nz_inner": 400, "nx_inner_boundary": 10,
               "nz_inner_boundary": 10, "dx": 1.249, "dz": 1.249, "dt": 0.0002},
    "boundary": {"np_boundary": 25, "np_factor": 0.015},
    "medium": {"scalar_rho": 1500.0, "scalar_vp": 2000.0, "scalar_vs": 800.0},
    "sources": {"peak_frequency": 50.0, "n_sources": 2, "n_shots": 1,
                "source_timeshift": 0.005, "delay_cycles_per_shot": 24,
                "moment_angles": [90, 180], "ix_sources": [150, 350], "iz_sources": [50, 50],
                "which_source_to_fire_in_which_shot": [[0, 1]]},
    "receivers": {"nr": 4, "ix_receivers": [50, 150, 250, 350],
                  "iz_receivers": [350, 350, 350, 350]},
    "inversion": {"snapshot_interval": 10},
    "basis": {"npx": 1, "npz": 1},
    "output": {"observed_data_folder": ".", "stf_folder": "."},
}


def get_dictionary():
    """The default configuration as a dict of sections (psvWave/__init__.py:34-97)."""
    return copy.deepcopy(_DEFAULTS)


def write_dictionary(filename, dictionary):
    """Write a configuration dict as INI, lists as {a, b} (psvWave/__init__.py:112-125)."""
    config = configparser.ConfigParser()
    for section, content in dictionary.items():
        config.add_section(section)
        for name, value in content.items():
            config.set(section, name, str(value).replace("[", "{").replace("]", "}"))
    with open(filename, "w") as f:
        config.write(f)


def from_dictionary(dictionary, filename="autogenerated.conf", **kwargs):
    """Write the dict to `filename` and build an fdModel from it
    (psvWave/__init__.py:103-109)."""
    from .model import fdModel

    write_dictionary(filename, dictionary)
    return fdModel(filename, **kwargs)


def to_parameters(dictionary):
    """Flatten a configuration dict into fdModel.from_parameters keywords."""
    out = {}
    for section in dictionary.values():
        out.update(section)
    return out
