"""The magnetisation (Bloch) walk: the reference's magAcquisition /
magAcquisitionStream API (src/acquisition/magAcquisition.cuh,
src/acquisition/magAcquisitionStream.cuh) and its B-field functors
(src/functors/bfunctors.cuh) over axx_run_mag.

Units are the reference's: lengths mm, times ms, B in T, G in T/mm.  The
reference fixes GAMMA at compile time (examples use 267500 for protons,
-203789 for helium-3, 73997 for neutrons); here it is a run parameter, and
the functors that use it (QSC_PGSE's and UCN_lowfield's RF amplitude and
frequency) take the run's value.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import List, Sequence

import numpy as np

from . import _native as N
from .acquisition import GAMMA, PI, Device, Vector3, default_device, linear_regression

ROTATE, RK4, ROTATE_MULTISTEP, DORP = 0, 1, 2, 3


def _vec(v):
    return (float(v[0]), float(v[1]), float(v[2]))


class _Field:
    kind = 0

    def record(self) -> N.Field:
        f = N.Field()
        f.kind = self.kind
        for k, v in self._members().items():
            setattr(f, k, v)
        return f

    def _members(self):
        return {}


class QSC_GRE(_Field):
    """Quadrupolar saddle coil, gradient echo (bfunctors.cuh:5-53)."""
    kind = 0

    def __init__(self, B0=0.0, G=0.0, gradientDuration=0.0, gradientSpacing=0.0):
        self.B0, self.G = float(B0), float(G)
        self.gradientDuration, self.gradientSpacing = float(gradientDuration), float(gradientSpacing)

    def _members(self):
        return dict(B0=self.B0, G=self.G, duration=self.gradientDuration,
                    spacing=self.gradientSpacing)

    def getB(self, gamma=GAMMA):
        return (self.G * self.G * self.gradientDuration ** 2 * gamma * gamma *
                ((2.0 / 3.0) * self.gradientDuration + self.gradientSpacing))

    def getDiffusionTime(self):
        return self.gradientSpacing + self.gradientDuration


class QSC_PGSE(QSC_GRE):
    """Saddle-coil PGSE with a refocusing RF pulse at TE/2 (:55-128)."""
    kind = 1

    def __init__(self, B0=0.0, G=0.0, gradientDuration=0.0, gradientSpacing=0.0, rfDuration=0.0,
                 dtmin=0.0, dtmax=0.0, TE=0.0):
        super().__init__(B0, G, gradientDuration, gradientSpacing)
        self.rfDuration, self.dtmin, self.dtmax, self.TE = (float(rfDuration), float(dtmin),
                                                            float(dtmax), float(TE))

    def _members(self):
        m = super()._members()
        m.update(rf_duration=self.rfDuration, dtmin=self.dtmin, dtmax=self.dtmax, TE=self.TE)
        return m

    def getStepTimeMin(self, time):
        return self.dtmin if (self.TE / 2.0 <= time < self.TE / 2.0 + self.rfDuration) else self.dtmax


class QSC_COS_GRE(_Field):
    """Saddle coil with cosine lobes (:130-195)."""
    kind = 2

    def __init__(self, B0=0.0, G=0.0, gradientDuration=0.0, gradientSpacing=0.0, numOfPeriods=1):
        self.B0, self.G = float(B0), float(G)
        self.gradientDuration, self.gradientSpacing = float(gradientDuration), float(gradientSpacing)
        self.numOfPeriods = int(numOfPeriods)
        self.period = self.gradientDuration / self.numOfPeriods

    def _members(self):
        return dict(B0=self.B0, G=self.G, duration=self.gradientDuration,
                    spacing=self.gradientSpacing, num_periods=self.numOfPeriods)

    def getB(self, gamma=GAMMA):
        return (gamma * gamma * 0.25 * self.G * self.G * self.gradientDuration ** 3 /
                (PI * PI * self.numOfPeriods * self.numOfPeriods))

    def getFreq(self):
        return 1.0 / self.period


class QSC_GRE_TRAP(_Field):
    """Saddle coil with trapezoidal lobes (:197-281); the ramps multiply the
    gradient field by (G / ramp) t as the reference writes them."""
    kind = 3

    def __init__(self, B0=0.0, G=0.0, gradientDuration=0.0, gradientSpacing=0.0,
                 gradientRampTime=0.0):
        self.B0, self.G = float(B0), float(G)
        self.gradientDuration, self.gradientSpacing = float(gradientDuration), float(gradientSpacing)
        self.gradientRampTime = float(gradientRampTime)

    def _members(self):
        return dict(B0=self.B0, G=self.G, duration=self.gradientDuration,
                    spacing=self.gradientSpacing, ramp=self.gradientRampTime)


class SIN_GRE(_Field):
    """z field B0 + (G . r) sin(2 pi t / period) per lobe (:283-331)."""
    kind = 4

    def __init__(self, B0=0.0, G=(0.0, 0.0, 0.0), gradientDuration=0.0, gradientSpacing=0.0,
                 period=0.0):
        self.B0, self.G = float(B0), Vector3(*_vec(G))
        self.gradientDuration, self.gradientSpacing = float(gradientDuration), float(gradientSpacing)
        self.period = float(period)

    def _members(self):
        return dict(B0=self.B0, gx=self.G.x, gy=self.G.y, gz=self.G.z,
                    duration=self.gradientDuration, spacing=self.gradientSpacing,
                    period=self.period)


class COS_GRE(_Field):
    """z field B0 + (G . r) cos(2 pi t / period), period = duration / N
    (:333-394); COS_GRE(B0, G, G_hat, duration, spacing, N) scales G_hat."""
    kind = 5

    def __init__(self, B0=0.0, G=(0.0, 0.0, 0.0), *args):
        if len(args) == 4:  # (B0, G, G_hat, duration, spacing, N)
            ghat, gd, gs, n = args
            g = Vector3(*(c * float(G) for c in _vec(ghat)))
            self.Gmag = float(G)
        else:
            gd, gs, n = args
            g = Vector3(*_vec(G))
            self.Gmag = math.sqrt(g.x ** 2 + g.y ** 2 + g.z ** 2)
        self.B0, self.G = float(B0), g
        self.gradientDuration, self.gradientSpacing = float(gd), float(gs)
        self.numOfPeriods = int(n)
        self.period = self.gradientDuration / self.numOfPeriods

    def _members(self):
        return dict(B0=self.B0, gx=self.G.x, gy=self.G.y, gz=self.G.z,
                    duration=self.gradientDuration, spacing=self.gradientSpacing,
                    num_periods=self.numOfPeriods)

    def getB(self, gamma=GAMMA):
        return (gamma * gamma * 0.25 * self.Gmag * self.Gmag * self.gradientDuration ** 3 /
                (PI * PI * self.numOfPeriods * self.numOfPeriods))

    def getFreq(self):
        return 1.0 / self.period


class RECT_GRE(_Field):
    """z field B0 +- G . r in the two lobes (:396-427)."""
    kind = 6

    def __init__(self, B0=0.0, G=(0.0, 0.0, 0.0), gradientDuration=0.0, gradientSpacing=0.0):
        self.B0, self.G = float(B0), Vector3(*_vec(G))
        self.gradientDuration, self.gradientSpacing = float(gradientDuration), float(gradientSpacing)

    def _members(self):
        return dict(B0=self.B0, gx=self.G.x, gy=self.G.y, gz=self.G.z,
                    duration=self.gradientDuration, spacing=self.gradientSpacing)


class UCN_lowfield(_Field):
    """Low-field ultracold-neutron cell: pi/2 RF pulse then a linear gradient
    (:429-476)."""
    kind = 7

    def __init__(self, B0=0.0, G=0.0, rfDuration=0.0, dtmin=0.0, dtmax=0.0):
        self.B0, self.G = float(B0), float(G)
        self.rfDuration, self.dtmin, self.dtmax = float(rfDuration), float(dtmin), float(dtmax)

    def _members(self):
        return dict(B0=self.B0, G=self.G, rf_duration=self.rfDuration, dtmin=self.dtmin,
                    dtmax=self.dtmax)

    def getStepTimeMin(self, time):
        return self.dtmin if time <= self.rfDuration else self.dtmax


class MagResult:
    """Per-field sums over walkers of the final magnetisation."""

    def __init__(self, mx, my, mz, n):
        self.mx, self.my, self.mz, self.n = mx, my, mz, int(n)

    @property
    def signal(self) -> np.ndarray:
        """|M_xy| / N per field."""
        return np.hypot(self.mx, self.my) / self.n


def _mag_params(num_walkers, steps, timestep, seed, m0, integrator, specular, gamma,
                walker_offset, fix_init_quirk, dorp_levels=0, dorp_tol=0.0):
    flags = (0 if specular else N.FLAG_SIMPLE_REJECTION) | (N.FLAG_FIX_INIT_QUIRK if fix_init_quirk else 0)
    return N.MagParams(int(num_walkers), int(steps), int(integrator), flags, int(dorp_levels),
                       int(seed) & 0xFFFFFFFFFFFFFFFF, float(timestep), float(gamma),
                       (C.c_double * 3)(*_vec(m0)), int(walker_offset), float(dorp_tol))


def run_mag(pore, fields: Sequence[_Field], num_walkers: int, steps: int, timestep: float,
            seed: int, *, m0=(1.0, 0.0, 0.0), integrator: int = ROTATE, specular: bool = True,
            gamma: float = GAMMA, walker_offset: int = 0, fix_init_quirk: bool = False,
            dorp_levels: int = 0, dorp_tol: float = 0.0, device: Device = None) -> MagResult:
    """One magnetisation walk (axx_run_mag): walkers start in `pore`, every
    field functor's magnetisation is summed over the walkers.  integrator
    DORP: adaptive Dormand-Prince with up to `dorp_levels` halvings of the
    step (0: 3) at tolerance `dorp_tol` (0: 1e-6)."""
    dev = device or default_device()
    nf = len(fields)
    f = N.array_of(N.Field, [q.record() for q in fields])
    p = _mag_params(num_walkers, steps, timestep, seed, m0, integrator, specular, gamma,
                    walker_offset, fix_init_quirk, dorp_levels, dorp_tol)
    out = [np.zeros(max(nf, 1)) for _ in range(3)]
    ptr = [o.ctypes.data_as(C.POINTER(C.c_double)) for o in out]
    N.check(N.lib().axx_run_mag(dev.h, C.byref(pore.record()), f, nf, C.byref(p), *ptr), dev.h)
    return MagResult(out[0][:nf], out[1][:nf], out[2][:nf], num_walkers)


def trace_mag(pore, fields: Sequence[_Field], num_trace: int, steps: int, timestep: float,
              seed: int, *, m0=(1.0, 0.0, 0.0), integrator: int = ROTATE,
              specular: bool = True, gamma: float = GAMMA, fix_init_quirk: bool = False,
              dorp_levels: int = 0, dorp_tol: float = 0.0, device: Device = None) -> dict:
    """The first num_trace walkers of the same walk: init_pos, pos, hits,
    words per move and the final magnetisation m [num_trace, nfield, 3]."""
    dev = device or default_device()
    nf = len(fields)
    f = N.array_of(N.Field, [q.record() for q in fields])
    p = _mag_params(num_trace, steps, timestep, seed, m0, integrator, specular, gamma, 0,
                    fix_init_quirk, dorp_levels, dorp_tol)
    n = num_trace * max(steps - 1, 0)
    ip = np.zeros(num_trace * 3, np.float32)
    pos = np.zeros(max(n, 1) * 3, np.float32)
    hits = np.zeros(max(n, 1), np.int32)
    words = np.zeros(max(n, 1), np.int32)
    m = np.zeros(num_trace * nf * 3, np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    ip32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
    N.check(N.lib().axx_trace_mag(dev.h, C.byref(pore.record()), f, nf, C.byref(p), num_trace,
                                  fp(ip), fp(pos), ip32(hits), ip32(words), fp(m)), dev.h)
    return dict(init_pos=ip.reshape(num_trace, 3),
                pos=pos[: n * 3].reshape(num_trace, steps - 1, 3),
                hits=hits[:n].reshape(num_trace, steps - 1),
                words=words[:n].reshape(num_trace, steps - 1),
                m=m.reshape(num_trace, nf, 3))


class magAcquisition:
    """magAcquisition<FieldType> (magAcquisition.cuh:1-86)."""

    def __init__(self, numOfMeas, numOfSteps, seed):
        self.numOfMeasurements = int(numOfMeas)
        self.numOfSteps = int(numOfSteps)
        self.seed = int(seed)
        self.mx = [0.0] * self.numOfMeasurements
        self.my = [0.0] * self.numOfMeasurements
        self.mz = [0.0] * self.numOfMeasurements
        self.fieldFunctors: List[_Field] = []
        self.ADC = 0.0
        self.ADCmeansquare = 0.0
        self.points = 0

    def addMeasurement(self, field):
        if len(self.fieldFunctors) >= self.numOfMeasurements:
            raise IndexError("more measurements than numOfMeas")
        self.fieldFunctors.append(field)

    def getFieldFunctors(self):
        return self.fieldFunctors

    def getMx(self):
        return self.mx

    def getMy(self):
        return self.my

    def getMz(self):
        return self.mz

    def getNumOfMeas(self):
        return self.numOfMeasurements

    def getNumOfSteps(self):
        return self.numOfSteps

    def getSeed(self):
        return self.seed

    def calcADC(self):
        """ADC from ln|M_xy| against b, running mean over repeats (:52-77)."""
        self.points += 1
        b = [f.getB() for f in self.fieldFunctors]
        ln = [math.log(math.sqrt(self.mx[i] ** 2 + self.my[i] ** 2))
              for i in range(self.numOfMeasurements)]
        adc = -1.0 * linear_regression(ln, b)
        if self.points == 1:
            self.ADC, self.ADCmeansquare = adc, adc * adc
        else:
            p = self.points
            self.ADC = (self.ADC * (p - 1) + adc) / p
            self.ADCmeansquare = (self.ADCmeansquare * (p - 1) + adc * adc) / p

    def getADC(self):
        return self.ADC

    def getADCError(self):
        return math.sqrt(max(self.ADCmeansquare - self.ADC * self.ADC, 0.0))


class magAcquisitionStream:
    """magAcquisitionStream<FieldType> (magAcquisitionStream.cuh:5-342): a
    set of acquisitions run on one walker population size."""

    def __init__(self, num):
        self.number_of_particles = int(num)
        self.acqSet: List[magAcquisition] = []
        self.steps_max = -1
        self.meas_max = -1

    def addAcquisition(self, acq: magAcquisition):
        self.acqSet.append(acq)
        self.steps_max = max(self.steps_max, acq.getNumOfSteps())
        self.meas_max = max(self.meas_max, acq.getNumOfMeas())

    def getAcquisition(self, num) -> magAcquisition:
        return self.acqSet[num]

    def runAcquisition(self, num, basis, initialM, timestep, blocks=None, threads=None,
                       devNum=None, numOfSM=None, *, integrator=ROTATE, specular=True,
                       gamma=GAMMA, device: Device = None):
        """runAcquisition(num, basis, initialM, timestep, ...) (:37-90); the
        launch-shape arguments are accepted and ignored."""
        acq = self.acqSet[num]
        fields = acq.getFieldFunctors()
        r = run_mag(basis, fields, self.number_of_particles, acq.getNumOfSteps(), timestep,
                    acq.getSeed(), m0=_vec(initialM), integrator=integrator, specular=specular,
                    gamma=gamma, device=device)
        acq.mx, acq.my, acq.mz = list(r.mx), list(r.my), list(r.mz)
        return r

    def runAcquisitionStream(self, basis, initialM, timestep, blocks=None, threads=None,
                             numOfDevices=1, plan=None, numOfSMPerDevice=None, *,
                             integrator=ROTATE, specular=True, gamma=GAMMA,
                             device: Device = None):
        """runAcquisitionStream (:142-319): every acquisition of the set."""
        return [self.runAcquisition(i, basis, initialM, timestep, integrator=integrator,
                                    specular=specular, gamma=gamma, device=device)
                for i in range(len(self.acqSet))]
