"""ctypes mirror of include/diffstir.h (structs, constants, prototypes)."""

import ctypes as C

DSTIR_OK = 0
DSTIR_EINVAL = -1
DSTIR_ENOMEM = -2
DSTIR_ECUDA = -3
DSTIR_ESTATE = -4
DSTIR_ERANGE = -5

DSTIR_STATUS_NAN = 1
DSTIR_STATUS_TIMEOUT = 4
DSTIR_STATUS_OUT_OF_GRID = 2

MODEL_CARREAU, MODEL_CROSS, MODEL_HB = 0, 1, 2
ROD_PARTICLES, ROD_CYLINDER = 0, 1
J_DET, J_SVD = 0, 1

_ERRNAMES = {
    DSTIR_EINVAL: 'DSTIR_EINVAL', DSTIR_ENOMEM: 'DSTIR_ENOMEM', DSTIR_ECUDA: 'DSTIR_ECUDA',
    DSTIR_ESTATE: 'DSTIR_ESTATE', DSTIR_ERANGE: 'DSTIR_ERANGE',
}


class DstirSceneDesc(C.Structure):
    _fields_ = [
        ('n_grid', C.c_int32),
        ('bound', C.c_int32),
        ('n_liquid', C.c_int32),
        ('n_rod', C.c_int32),
        ('n_container', C.c_int32),
        ('model', C.c_int32),
        ('rod_mode', C.c_int32),
        ('j_mode', C.c_int32),
        ('container_wall', C.c_int32),
        ('reserved', C.c_int32),
        ('dt', C.c_float),
        ('gravity', C.c_float),
        ('bulk_modulus', C.c_float),
        ('liquid_p_vol', C.c_float),
        ('liquid_p_mass', C.c_float),
        ('rod_p_mass', C.c_float),
        ('container_p_mass', C.c_float),
        ('force_scale', C.c_float),
        ('container_cx', C.c_float),
        ('container_cz', C.c_float),
        ('container_r', C.c_float),
        ('rod_radius', C.c_float),
    ]


# name -> (restype, argtypes); every symbol include/diffstir.h declares
P = C.c_void_p
PROTOTYPES = {
    'dstir_create': (C.c_int, [C.POINTER(DstirSceneDesc), C.c_int32, C.c_int32, C.POINTER(P)]),
    'dstir_destroy': (None, [P]),
    'dstir_last_error': (C.c_char_p, [P]),
    'dstir_num_particles': (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    'dstir_set_state': (C.c_int, [P, P, P, P, P, P]),
    'dstir_get_state': (C.c_int, [P, P, P, P, P, P]),
    'dstir_set_params': (C.c_int, [P, P, P, P]),
    'dstir_set_trajectory': (C.c_int, [P, P, P]),
    'dstir_forward': (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P]),
    'dstir_substep': (C.c_int, [P, C.c_int32, P, P]),
    'dstir_backward': (C.c_int, [P, P, P, P, P, P, P, P]),
    'dstir_status': (C.c_int, [P, C.POINTER(C.c_uint32), P]),
    'dstir_set_option': (C.c_int, [P, C.c_char_p, C.c_int64]),
    'dstir_get_option': (C.c_int, [P, C.c_char_p, C.POINTER(C.c_int64)]),
    'dstir_svd3': (C.c_int, [P, P, P, P, C.c_int64, P]),
    'dstir_svd3_backward': (C.c_int, [P, P, P, P, P, P, P, C.c_int64, P]),
    'dstir_substep_static': (C.c_int, [C.POINTER(DstirSceneDesc), P, P, P, P, P, P]),
    'dstir_measure_red_rate': (C.c_int, [C.c_int64, C.c_int32, C.POINTER(C.c_double), P]),
    'dstir_measure_fp32_rate': (C.c_int, [C.c_int32, C.POINTER(C.c_double), P]),
}


def bind(lib):
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def errname(code):
    return _ERRNAMES.get(code, str(code))
