"""Writers of BEEP's posterior sample files, for trajectories sampled on the
GPU (the particle filter's lineage, MBP chain states).

The files are the reference's own format, byte for byte:
  * ``sample<k>_parameter.csv``  -- ``State::save`` (src/state.cc:709-739):
    ``Parameter,Value``, ``Error function,<EF>``, then ``<name>,<value>`` per
    parameter;
  * ``sample<k>_transition.csv`` -- the same function: ``Time,Transitions
    (ordered by area x trans x democatpos)``, then per step the division time
    and the counts in area, transition, dp order;
  * ``sample_information.txt``   -- ``Mpi::gather_samples`` (src/mpi.cc:706-716).
Numbers are printed as a C++ stream prints a double by default (6
significant digits, %g style).  Division times are (s + 1/2) period /
ndivision, plus the start time when times are numbers (src/details.cc:102-106).
"""
from __future__ import annotations

import os
from typing import Sequence

import numpy as np


def fmt(x: float) -> str:
    """A double as ``std::ostream << x`` prints it with the default precision (6, %g)."""
    return "%g" % float(x)


def division_times(period: int, ndivision: int, start: float = 0.0, numeric_time: bool = True) -> np.ndarray:
    s = np.arange(ndivision, dtype=np.float64)
    t = (s + 0.5) * float(period) / float(ndivision)
    return t + float(start) if numeric_time else t


def write_sample(directory: str, index: int, EF: float, param_names: Sequence[str], paramval: Sequence[float],
                 transnum: np.ndarray, times: Sequence[float]) -> None:
    """Writes sample<index>_parameter.csv and sample<index>_transition.csv.

    transnum: [ndivision][narea][ntrans][ndemocatpos] counts of the sample."""
    if len(param_names) != len(paramval):
        raise ValueError("one name per parameter value")
    tn = np.asarray(transnum)
    if tn.ndim != 4 or tn.shape[0] != len(times):
        raise ValueError("transnum must be [ndivision][narea][ntrans][ndemocatpos] with one time per step")
    base = os.path.join(directory, f"sample{index}")
    with open(base + "_parameter.csv", "w", newline="") as f:
        f.write("Parameter,Value\n")
        f.write(f"Error function,{fmt(EF)}\n")
        for name, v in zip(param_names, paramval):
            f.write(f"{name},{fmt(v)}\n")
    flat = tn.reshape(tn.shape[0], -1)
    with open(base + "_transition.csv", "w", newline="") as f:
        f.write("Time,Transitions (ordered by area x trans x democatpos)\n")
        for s in range(flat.shape[0]):
            f.write(fmt(times[s]))
            f.write("".join("," + fmt(v) for v in flat[s]))
            f.write("\n")


def write_sample_information(directory: str, nsamples: int, toml_file: str, start: str, end: str,
                             division_per_time: int, ndivision: int) -> None:
    """sample_information.txt of a set of samples (Mpi::gather_samples)."""
    with open(os.path.join(directory, "sample_information.txt"), "w", newline="") as f:
        f.write(f"# Samples = '{nsamples}'\n")
        f.write(f"TOML file = '{toml_file}'\n")
        f.write(f"start = '{start}'\n")
        f.write(f"end = '{end}'\n")
        f.write(f"division_per_time = '{division_per_time}'\n")
        f.write(f"timesteps = '{ndivision}'\n")
