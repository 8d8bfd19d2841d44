"""GB300-native finite-element assembly path (Tianxin/Panzer drop-in).

The compute path is libtianxin_gb300.so (hand-written sm_103a kernels behind
the C-ABI in include/tianxin_gb300.h); this package is its Python host side.
"""
from . import _abi
from ._abi import (ALL_SIDES, SIDE_XMAX, SIDE_XMIN, SIDE_YMAX, SIDE_YMIN, SIDE_ZMAX, SIDE_ZMIN, TX_HCURL_I1,
                   TX_HGRAD_C1, TX_HGRAD_C2, TX_PHYS_ELASTICITY, TX_PHYS_HEAT, TX_PHYS_MAXWELL, TX_PHYS_POISSON,
                   TX_SOURCE_AFFINE, TX_SOURCE_CONST, TX_SOURCE_SINE, TX_TOPO_HEX, TX_TOPO_TET, equation_set,
                   mesh_desc)
from ._lib import TxError, load
from .panzer import (HEX, TET, AssemblyEngine, Batch, ip_coordinates, ExodusReaderFactory, ExplicitConnManager, exodus_summary, BlockedCrsMatrix, BlockedDOFManager, BlockedModelEvaluator,
                     BlockedTpetraLinearObjFactory, CapturedGraph, CartesianConnManager, CrsMatrix, DirichletBC, DOFManager,
                     HostEvaluator, ModelEvaluator, NeumannBC, Response, TpetraLinearObjFactory, neumann_value,
                     synchronize)

__all__ = ["CartesianConnManager", "DOFManager", "TpetraLinearObjFactory", "CrsMatrix", "DirichletBC",
           "NeumannBC", "neumann_value", "Response", "ip_coordinates", "CapturedGraph", "HostEvaluator", "AssemblyEngine", "ModelEvaluator", "ExodusReaderFactory", "ExplicitConnManager", "exodus_summary", "BlockedDOFManager", "BlockedTpetraLinearObjFactory", "BlockedCrsMatrix",
           "BlockedModelEvaluator", "TxError", "load", "equation_set", "mesh_desc", "synchronize"]
