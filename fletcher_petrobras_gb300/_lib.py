"""ctypes binding of libfletcher_gb300.so (include/fletcher_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB as _LIB_PATH, build as _do_build

_LIB = None

FP = C.POINTER(C.c_float)
DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)

# name -> (restype, argtypes); every symbol declared in include/fletcher_gb300.h.
SIGNATURES = {
    "DRIVER_Initialize": (None, [C.c_int] * 4 + [C.c_float] * 4 + [FP] * 10),
    "DRIVER_Finalize": (None, []),
    "DRIVER_Propagate": (None, [C.c_int] * 4 + [C.c_float] * 4 + [C.c_int] + [FP] * 4),
    "DRIVER_Update_pointers": (None, [C.c_int] * 3 + [FP]),
    "DRIVER_InsertSource": (None, [C.c_float, C.c_int, C.c_int, FP, FP, C.c_float]),
    "FLETCHER_SetErrorMode": (None, [C.c_int]),
    "FLETCHER_GetLastError": (C.c_int, []),
    "FLETCHER_GetLastErrorString": (C.c_char_p, []),
    "FLETCHER_ClearError": (None, []),
    "FLETCHER_SetStream": (C.c_int, [C.c_void_p]),
    "FLETCHER_GetStream": (C.c_void_p, []),
    "FLETCHER_SetForm": (C.c_int, [C.c_int]),
    "FLETCHER_SetNumerics": (C.c_int, [C.c_int]),
    "FLETCHER_SetCoefLayout": (C.c_int, [C.c_int]),
    "FLETCHER_CoefLayout": (C.c_int, []),
    "FLETCHER_InitPhases": (C.c_int, [DP]),
    "FLETCHER_DebugPoisonPadding": (C.c_int, [C.c_float]),
    "FLETCHER_InjectFault": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "FLETCHER_SetHostAccess": (C.c_int, [C.c_int]),
    "FLETCHER_HostAccess": (C.c_int, []),
    "FLETCHER_SetTileConfig": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "FLETCHER_Run": (C.c_int, [C.c_int, C.c_long, FP]),
    "FLETCHER_Synchronize": (C.c_int, []),
    "FLETCHER_GetField": (C.c_int, [C.c_int, FP]),
    "FLETCHER_GetCoefficients": (C.c_int, [FP]),
    "FLETCHER_KernelLaunches": (C.c_long, []),
    "FLETCHER_DeviceBytes": (C.c_size_t, []),
    "FLETCHER_BytesPerCell": (C.c_double, []),
    "FLETCHER_ReadFieldNoAlloc": (C.c_int, [C.c_void_p] + [C.c_int] * 5 + [FP]),
    "FLETCHER_BatchCreate": (C.c_int, [C.c_int] + [C.c_float] * 4),
    "FLETCHER_BatchAddShot": (C.c_int, [C.c_int] * 3 + [FP, C.c_long, C.c_int]),
    "FLETCHER_BatchSetTileConfig": (C.c_int, [C.c_int, C.c_int]),
    "FLETCHER_BatchRun": (C.c_int, [FP, C.c_int, C.c_int, FP]),
    "FLETCHER_BatchSetChains": (C.c_int, [C.c_int]),
    "FLETCHER_BatchLastChains": (C.c_int, []),
    "FLETCHER_BatchReset": (C.c_int, []),
    "FLETCHER_BatchGetField": (C.c_int, [C.c_int, C.c_int, FP]),
    "FLETCHER_BatchInfo": (C.c_int, [C.POINTER(C.c_long), DP, C.POINTER(C.c_long), C.POINTER(C.c_size_t)]),
    "FLETCHER_BatchDestroy": (None, []),
    "FLETCHER_ModelHomogeneous": (None, [C.c_long] + [C.c_float] * 6 + [FP]),
    "FLETCHER_ModelLayered": (None, [C.c_int] * 6 + [C.c_uint64] + [C.c_float] * 3 + [FP, IP]),
    "FLETCHER_RandomVelocityBoundary": (None, [C.c_int] * 8 + [FP, FP, C.c_uint]),
    "FLETCHER_Source": (C.c_float, [C.c_float, C.c_int, C.c_double]),
    "FLETCHER_RecommendedDt": (C.c_float, [C.c_long, FP, FP, C.c_float, C.c_float, C.c_float]),
    "FLETCHER_Model": (C.c_int, [C.c_int, C.c_long, C.c_double, C.c_float] + [C.c_int] * 4 + [C.c_float] * 4
                       + [FP] * 10 + [DP]),
    "FLETCHER_Autotune": (C.c_int, [C.c_char_p, C.c_int]),
    "FLETCHER_GetTileConfig": (C.c_int, [IP, IP]),
    "FLETCHER_ModelPhases": (None, [DP]),
    "FLETCHER_TuneConfigLookup": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_int, IP, IP]),
    "FLETCHER_TuneConfigStore": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "FLETCHER_SnapshotBegin": (C.c_int, [C.c_int, FP]),
    "FLETCHER_SnapshotWait": (C.c_int, []),
    "FLETCHER_PinHost": (C.c_int, [C.c_void_p, C.c_size_t]),
    "FLETCHER_UnpinHost": (C.c_int, [C.c_void_p]),
    "FLETCHER_DumpFieldToFile": (C.c_int, [C.c_int] * 9 + [C.c_float] * 3 + [FP, C.c_char_p]),
    "FLETCHER_OpenSliceFile": (C.c_void_p, [C.c_int] * 6 + [C.c_float] * 4 + [C.c_char_p]),
    "FLETCHER_DumpSliceFile": (C.c_int, [C.c_int] * 3 + [FP, C.c_void_p]),
    "FLETCHER_SliceAppend": (C.c_int, [C.c_void_p, C.c_int]),
    "FLETCHER_CloseSliceFile": (C.c_int, [C.c_void_p]),
    "FLETCHER_SliceFrames": (C.c_int, [C.c_void_p]),
    "FLETCHER_DumpSliceSummary": (C.c_int, [C.c_int] * 3 + [C.c_void_p, C.c_float, C.c_int, FP, C.c_float]),
    "FLETCHER_AbcInit": (C.c_int, [C.c_uint]),
    "FLETCHER_AbcSetWeights": (C.c_int, [FP]),
    "FLETCHER_AbcGetWeights": (C.c_int, [FP]),
    "FLETCHER_AbcReserve": (C.c_int, [C.c_long]),
    "FLETCHER_AbcCollect": (C.c_int, [IP, IP, C.c_int, C.c_float, C.c_uint, C.c_float]),
    "FLETCHER_AbcSamples": (C.c_long, []),
    "FLETCHER_AbcGetSamples": (C.c_int, [C.c_long, C.c_long, FP, FP, IP]),
    "FLETCHER_AbcTrain": (C.c_int, [C.c_int, C.c_int, C.c_float, C.c_uint, C.c_float, FP]),
    "FLETCHER_AbcGradient": (C.c_int, [FP, FP, C.c_int, FP, FP]),
    "FLETCHER_AbcForward": (C.c_int, [FP, C.c_int, FP]),
    "FLETCHER_SetBoundary": (C.c_int, [C.c_int, C.c_int, C.c_float]),
    "FLETCHER_PlanSegments": (C.c_int, [C.c_int] * 7 + [IP, C.c_int, IP, C.POINTER(C.c_long)]),
    "FLETCHER_AbcLayerCells": (C.c_long, []),
    "FLETCHER_AbcSetInterval": (C.c_int, [C.c_int]),
    "FLETCHER_AbcRelease": (None, []),
}


def lib_path() -> str:
    return _LIB_PATH


def load(build_if_missing: bool = True):
    """Loads the library; fails loudly when it is missing and cannot be built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libfletcher_gb300.so not built ({path}); run fletcher_petrobras_gb300.build")
        _do_build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    lib.FLETCHER_SetErrorMode(1)  # record and return: the Python layer raises
    _LIB = lib
    return lib


def fptr(a):
    return a.ctypes.data_as(FP) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(IP) if a is not None else None
