"""Global values of a step and the ResultWriter output, from the per-step
records of ``Engine.run`` (Upot, virial, sum m v^2, sum I w^2).

``global_values`` follows Domain::calculateGlobalValues for one thermostat
(src/Domain.cpp:157-345): Upot and virial plus the long-range corrections,
T = (sum m v^2 + sum I w^2) / (3 N + rotDOF), the velocity-scaling betas
(beta_trans = (3 N T_target / sum m v^2)^0.4, beta_rot = (rotDOF T_target /
sum I w^2)^0.4, 1 without a target), and Domain::getGlobalPressure
(src/Domain.cpp:142-146): p = T rho + rho (virial / N) / 3 with
rho = N / (Lx Ly Lz) (Domain::evaluateRho).  The explosion heuristic of the thermostat is not
restated here; the engine applies it on the device and ``Engine.thermostat_betas``
reports the betas it used.

``ResultWriter`` writes ``<prefix>.res`` like io/ResultWriter.cpp:
a header, then every ``write_frequency`` steps the step, time, U_pot and its
sliding average, U_kin = (sum m v^2 + sum I w^2) / 2 and its average, p and
its average, the betas, c_v and N, each column ``write_precision + 15`` wide
in scientific notation.  The averages are utils/Accumulator.h windows of
``accumulation_steps`` entries summed in storage order, as the reference
sums them.  Domain::cv is 0 unless a checkpoint carried fluctuation sums,
which the engine does not read, so c_v is written as 0.
"""
from __future__ import annotations

import datetime
from dataclasses import dataclass
from typing import Optional

import numpy as np


@dataclass
class GlobalValues:
    upot: float
    virial: float
    temperature: float
    pressure: float
    ukin: float
    beta_trans: float
    beta_rot: float
    n: int


def system_constants(ps):
    """(N, total rotational degrees of freedom, box lengths) of a phase space."""
    dof = np.array([c.mass_inertia()[2] for c in ps.components], np.int64)
    return ps.n, int(dof[ps.comp].sum()), np.asarray(ps.box, float)


def global_values(record, n: int, rot_dof: int, box, target_temperature: Optional[float] = None,
                  upot_corr: float = 0.0, virial_corr: float = 0.0) -> GlobalValues:
    """One step's global values from its record (Upot, virial, sum m v^2,
    sum I w^2) as Domain::calculateGlobalValues forms them."""
    upot_l, vir_l, summv2, sumiw2 = (float(x) for x in record[:4])
    sumiw2 = sumiw2 if rot_dof > 0 else 0.0
    upot = upot_l + upot_corr
    virial = vir_l + virial_corr
    temperature = (summv2 + sumiw2) / float(3 * n + rot_dof) if n > 0 else (target_temperature or 0.0)
    bt = br = 1.0
    if target_temperature is not None and target_temperature > 0.0 and n > 0:
        bt = (3.0 * n * target_temperature / summv2) ** 0.4
        br = 1.0 if sumiw2 == 0.0 else (rot_dof * target_temperature / sumiw2) ** 0.4
    rho = n / (float(box[0]) * float(box[1]) * float(box[2]))  # Domain::evaluateRho
    pressure = temperature * rho + rho * (virial / n) / 3.0
    ukin = 0.5 * summv2 + 0.5 * sumiw2
    return GlobalValues(upot, virial, temperature, pressure, ukin, bt, br, n)


class Accumulator:
    """Sliding window of utils/Accumulator.h: a ring of ``window`` entries,
    averaged in storage order."""

    def __init__(self, window: int = 1000):
        self.data = np.zeros(window)
        self.window = window
        self.pos = 0
        self.size = 0

    def add(self, value: float):
        self.data[self.pos] = value
        self.pos = (self.pos + 1) % self.window
        self.size = min(self.size + 1, self.window)

    def average(self) -> float:
        s = 0.0
        for i in range(self.size):
            s += float(self.data[i])
        return s / self.size


class ResultWriter:
    """io/ResultWriter.cpp (readXML settings as arguments; init writes the
    header, end_step adds a step and writes its line every write_frequency
    steps, finish writes the closing comment)."""

    def __init__(self, output_prefix: str = "results", write_frequency: int = 1000, accumulation_steps: int = 1000,
                 write_precision: int = 5):
        if write_frequency <= 0:
            raise ValueError("write frequency must be a positive nonzero integer")
        self.prefix = output_prefix
        self.freq = write_frequency
        self.precision = write_precision
        self.width = write_precision + 15
        self.upot_acc = Accumulator(accumulation_steps)
        self.ukin_acc = Accumulator(accumulation_steps)
        self.p_acc = Accumulator(accumulation_steps)

    @property
    def path(self) -> str:
        return self.prefix + ".res"

    def init(self):
        now = datetime.datetime.now().strftime("%c")
        cols = ["time", "U_pot", "U_pot_avg", "U_kin", "U_kin_avg", "p", "p_avg", "beta_trans", "beta_rot", "c_v",
                "N"]
        with open(self.path, "w") as f:
            f.write(f"# ls1 MarDyn simulation started at {now}\n")
            f.write(f"# Averages are the accumulated values over {self.upot_acc.window} time steps.\n")
            f.write("# step".rjust(10) + "".join(c.rjust(self.width) for c in cols) + "\n")

    def _num(self, v: float) -> str:
        return ("%.*e" % (self.precision, v)).rjust(self.width)

    def end_step(self, step: int, time: float, g: GlobalValues, cv: float = 0.0):
        self.upot_acc.add(g.upot)
        self.ukin_acc.add(g.ukin)
        self.p_acc.add(g.pressure)
        if step % self.freq != 0:
            return
        line = str(step).rjust(10)
        for v in (time, g.upot, self.upot_acc.average(), g.ukin, self.ukin_acc.average(), g.pressure,
                  self.p_acc.average(), g.beta_trans, g.beta_rot, cv):
            line += self._num(v)
        line += str(int(g.n)).rjust(self.width)
        with open(self.path, "a") as f:
            f.write(line + "\n")

    def finish(self):
        now = datetime.datetime.now().strftime("%c")
        with open(self.path, "a") as f:
            f.write(f"# ls1 mardyn simulation finished at {now}\n")


def write_results(prefix: str, records: np.ndarray, n: int, rot_dof: int, box, dt: float,
                  first_step: int = 1, start_time: float = 0.0, target_temperature: Optional[float] = None,
                  upot_corr: float = 0.0, virial_corr: float = 0.0, write_frequency: int = 1000,
                  accumulation_steps: int = 1000, write_precision: int = 5) -> ResultWriter:
    """ResultWriter output of the rows of ``Engine.run``: row k is step
    first_step + k, the time advanced by dt per step from start_time (the
    repeated addition of Simulation::advanceSimulationTime)."""
    rw = ResultWriter(prefix, write_frequency, accumulation_steps, write_precision)
    rw.init()
    t = start_time
    for k, row in enumerate(records):
        t += dt
        g = global_values(row, n, rot_dof, box, target_temperature, upot_corr, virial_corr)
        rw.end_step(first_step + k, t, g)
    return rw
