"""``import NexusMD`` for scripts written against the reference's SWIG module;
the implementation is nexusmd_gb300.NexusMD (CUDA engine behind a C ABI)."""
from nexusmd_gb300.NexusMD import *  # noqa: F401,F403
from nexusmd_gb300.NexusMD import (AngleParams, BondParams, Coords3D, NonbondedParams,  # noqa: F401
                                   PTorsionParams, StateXMLParser, SystemXMLParser, TaskDispatcher)
