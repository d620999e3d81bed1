"""GB300-native statevector engine for q1tsim.

The engine replaces q1tsim's coefficient-vector backend (`VectorState`
behind the `QuState` trait, src/qustate.rs:5-89) with hand-written sm_103a
CUDA kernels reached through a C ABI (include/q1gpu.h, libq1gpu.so).
"""
from . import gates
from ._lib import (DeviceError, DeviceTimeout, InvalidArgument, InvalidCBit, InvalidNrBits,
                   InvalidNrControlBits, InvalidNrMeasurementBits, InvalidQBit, NotEnoughSpace,
                   NotExecuted, OutOfMemory, Q1Error)
from .circuit import Circuit
from .vectorstate import Plan, Rng, VectorState, device_info

__all__ = ["gates", "Circuit", "VectorState", "Plan", "Rng", "device_info", "Q1Error",
           "InvalidNrBits", "InvalidQBit", "InvalidCBit", "InvalidNrControlBits",
           "InvalidNrMeasurementBits", "NotEnoughSpace", "NotExecuted", "InvalidArgument",
           "OutOfMemory", "DeviceError", "DeviceTimeout"]
