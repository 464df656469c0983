"""ctypes binding of libvk_gb300.so (declared in include/vk_ros2.h).

The library is built in-tree by ``vulcan_gb300._build.build()``.  Loading
fails loudly when it is missing: there is no CPU fallback for the step.
"""
from __future__ import annotations

import ctypes as C
import os


from ._build import LIB

VK_OK, VK_EINVAL, VK_ECUDA, VK_ESINGULAR, VK_ENAN, VK_EMAXATTEMPT, VK_ETIMEOUT, VK_ENOMEM = range(8)
VK_PREC_FP64, VK_PREC_MIXED = 0, 1
VK_F_MOLDIFF, VK_F_TOPFLUX, VK_F_BOTFLUX = 1, 2, 4
VK_TUNE_LU32, VK_TUNE_LU64, VK_TUNE_SWEEP64, VK_TUNE_REFINE = 0, 1, 2, 3
LU32_TILING_CAP = (48, 80, 112, 160, 128, 128)  # species each LU32 variant covers
LU32_TC = 4                                # the tensor-core factorisation (k_lu_tc)
LU32_TC_COOP = 5                           # the same, four warps per panel
(ATM_M, ATM_N0, ATM_TCO, ATM_G, ATM_DZI, ATM_KZZ, ATM_VZ, ATM_TI, ATM_HPI, ATM_HP,
 ATM_PICO, ATM_PICOU, ATM_DZ) = range(13)
ATM_NF = 13
SP_MS, SP_ALPHA, SP_TOPFLUX, SP_BOTFLUX, SP_BOTVDEP = range(5)
SP_NF = 5
MAX_NATOM = 16
NCOUNTERS = 6   # attempts, delta/negative/loss rejections, FP64 redo, accepted steps

_ERRNAMES = {1: 'VK_EINVAL', 2: 'VK_ECUDA', 3: 'VK_ESINGULAR', 4: 'VK_ENAN',
             5: 'VK_EMAXATTEMPT', 6: 'VK_ETIMEOUT', 7: 'VK_ENOMEM'}

# Every entry point include/vk_ros2.h declares.
EXPORTS = ('vk_network_compile', 'vk_network_info', 'vk_network_jac_pattern', 'vk_network_eval_host',
           'vk_network_free', 'vk_create', 'vk_destroy', 'vk_last_error',
           'vk_set_precision', 'vk_set_route', 'vk_set_columns', 'vk_update_state', 'vk_update_atm',
           'vk_update_k', 'vk_ros2_attempt', 'vk_set_atom_ini', 'vk_set_column_info',
           'vk_run', 'vk_run_budget', 'vk_get_state', 'vk_set_clock', 'vk_get_counters', 'vk_get_timing',
           'vk_network_last_error', 'vk_chem_source', 'vk_get_lhs',
           'vk_block_solve_noalloc', 'vk_get_refine_stats', 'vk_mlp_forward',
           'vk_mlp_backward', 'vk_mlp_adam', 'vk_get_conv', 'vk_set_rate_params',
           'vk_compute_k', 'vk_get_k', 'vk_photo_setup', 'vk_photo_reset',
           'vk_photo_update', 'vk_photo_get', 'vk_photo_set_cross_T', 'vk_set_rate_caps',
           'vk_set_launch', 'vk_get_launch', 'vk_set_conv_ignore', 'vk_get_lu32', 'vk_rhs',
           'vk_set_columns_slotted', 'vk_refill', 'vk_group_create', 'vk_group_run',
           'vk_group_timing', 'vk_group_destroy')


class VkNetworkDesc(C.Structure):
    _fields_ = [('ni', C.c_int), ('npair', C.c_int),
                ('reac_ptr', C.POINTER(C.c_int)), ('reac_sp', C.POINTER(C.c_int)),
                ('reac_nu', C.POINTER(C.c_int)),
                ('prod_ptr', C.POINTER(C.c_int)), ('prod_sp', C.POINTER(C.c_int)),
                ('prod_nu', C.POINTER(C.c_int)),
                ('natom', C.c_int), ('compo', C.POINTER(C.c_double))]


class VkCtrl(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        'rtol', 'atol', 'mtol', 'mtol_conv', 'pos_cut', 'nega_cut', 'loss_eps',
        'dt_min', 'dt_max', 'dt_var_min', 'dt_var_max',
        'yconv_cri', 'slope_cri', 'yconv_min', 'st_factor', 'trun_min', 'runtime')] + \
        [(n, C.c_int) for n in ('conv_step', 'count_min', 'count_max', 'update_frq',
                                'max_attempts', 'flags')] + \
        [('gs', C.c_double), ('Rp', C.c_double), ('flux_cri', C.c_double)]


class VkError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__('%s: %s' % (_ERRNAMES.get(code, str(code)), msg))
        self.code = code


_lib = None


def lib(path=None):
    """Load libvk_gb300.so once (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get('VK_GB300_LIB', LIB)
    if not os.path.exists(path):
        raise RuntimeError('libvk_gb300.so not found at %s: build it with '
                           'vulcan_gb300._build.build() (there is no CPU fallback)' % path)
    L = C.CDLL(path)
    P = C.POINTER
    d, i, vp = C.c_double, C.c_int, C.c_void_p
    pd, pi = P(d), P(i)
    sig = {
        'vk_network_compile': (i, [P(VkNetworkDesc), P(vp)]),
        'vk_network_info': (i, [vp, pi, pi, pi]),
        'vk_network_jac_pattern': (i, [vp, pi, pi]),
        'vk_network_eval_host': (i, [vp, P(C.c_double), P(C.c_double), d, P(C.c_double), P(C.c_double)]),
        'vk_network_free': (None, [vp]),
        'vk_network_last_error': (C.c_char_p, []),
        'vk_create': (i, [vp, i, i, i, P(vp)]),
        'vk_destroy': (None, [vp]),
        'vk_last_error': (C.c_char_p, [vp]),
        'vk_set_precision': (i, [vp, i, i, d]),
        'vk_set_route': (i, [vp, d]),
        'vk_set_columns': (i, [vp, i, pi, pd, pd, pd, pd, pd, pd]),
        'vk_update_state': (i, [vp, pd, pd]),
        'vk_update_atm': (i, [vp, pd]),
        'vk_update_k': (i, [vp, pd]),
        'vk_ros2_attempt': (i, [vp, pd, i, pd, pd, pd, pd, pd]),
        'vk_set_atom_ini': (i, [vp, pd]),
        'vk_set_column_info': (i, [vp, pi, pi]),
        'vk_set_conv_ignore': (i, [vp, pi]),
        'vk_get_lu32': (i, [vp, P(C.c_float)]),
        'vk_rhs': (i, [vp, pd, i, pd]),
        'vk_set_columns_slotted': (i, [vp, i, i, pi, pd, pd, pd, pd, pd, pd]),
        'vk_refill': (i, [vp, i, pi, pi, pd, pd, pd, pd, pd, pd, pd, pi, pi]),
        'vk_run': (i, [vp, P(VkCtrl), i, d]),
        'vk_run_budget': (i, [vp, P(VkCtrl), i, i, d]),
        'vk_group_create': (i, [P(vp), i, P(vp)]),
        'vk_group_run': (i, [vp, P(VkCtrl), i, i, d]),
        'vk_group_timing': (i, [vp, pd, pi]),
        'vk_group_destroy': (None, [vp]),
        'vk_get_state': (i, [vp, pd, pd, pd, pd, pi, pi, pd]),
        'vk_set_clock': (i, [vp, pd, pd, pi]),
        'vk_get_counters': (i, [vp, pi]),
        'vk_get_conv': (i, [vp, pd, pd]),
        'vk_set_rate_params': (i, [vp, pi, pi, pd, pd]),
        'vk_compute_k': (i, [vp]),
        'vk_set_rate_caps': (i, [vp, pi, pd, pd]),
        'vk_set_launch': (i, [vp, i, i, i]),
        'vk_get_launch': (i, [vp, i, pi, pi]),
        'vk_get_k': (i, [vp, pd]),
        'vk_photo_setup': (i, [vp, i, pd, pd, i, pi, pi, pd, i, pi, pd, i, pi, pd, pd,
                               C.c_double, C.c_double, C.c_double, C.c_double]),
        'vk_photo_reset': (i, [vp]),
        'vk_photo_update': (i, [vp, pi, pd]),
        'vk_photo_get': (i, [vp, pd, pd, pd]),
        'vk_photo_set_cross_T': (i, [vp, i, pi, pd, i, pi, pd]),
        'vk_get_timing': (i, [vp, pd, pd, pd, pd, pi]),
        'vk_chem_source': (i, [vp, pd, pd]),
        'vk_get_lhs': (i, [vp, pd, pd, pd, pd]),
        'vk_block_solve_noalloc': (i, [i, i, vp, vp, vp, vp, vp, vp]),
        'vk_get_refine_stats': (i, [vp, pi, pi]),
        'vk_mlp_forward': (i, [i, i, i, vp, vp, P(C.c_float), P(C.c_float), vp, i, vp]),
        'vk_mlp_backward': (i, [i, i, i, vp, vp, P(C.c_float), P(C.c_float), i, vp,
                                P(C.c_float), P(C.c_float), P(C.c_float), vp]),
        'vk_mlp_adam': (i, [C.c_longlong, P(C.c_float), vp, P(C.c_float), P(C.c_float),
                            P(C.c_float), C.c_float, C.c_float, C.c_float, C.c_float, i, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def ptr(a, ctype=C.c_double):
    """Pointer to a C-contiguous numpy array (or NULL for None)."""
    if a is None:
        return None
    assert a.flags['C_CONTIGUOUS'], 'array must be C-contiguous'
    return a.ctypes.data_as(C.POINTER(ctype))


def check(rc, handle=None):
    if rc != VK_OK:
        L = lib()
        msg = L.vk_last_error(handle)
        raise VkError(rc, msg.decode() if msg else '')
