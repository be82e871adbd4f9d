"""GB300-native (sm_103a) 3D channel-flow time step of chandc/F90_DNS.

The step of ``DNS_pressure_BC_3D.f90`` (rotational nonlinear term with
optional 2/3 filter, Crank-Nicolson Helmholtz solve with Kim & Moin wall
conditions, Galerkin pressure Poisson solve and projection, constant dp/dx or
PI bulk-velocity control) runs on one GPU behind the C-ABI declared in
``include/dns3d_capi.h``; :mod:`f90_dns_gb300.capi` binds it from Python.
"""
from .capi import (  # noqa: F401
    Batch,
    ChannelDNS,
    Dns3DError,
    Ensemble,
    Server,
    Diagnostics,
    config_from,
    default_config,
    footprint_bytes,
    load_library,
    read_namelist,
)
