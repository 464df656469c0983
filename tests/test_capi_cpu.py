"""C-ABI library: loads, exports every declared entry point, compiles networks
(host-only calls; nothing here launches device work)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import REPO
from helpers import golden, network, oracle_net
from oracle import ros2 as O


@pytest.fixture(scope='module')
def lib():
    from vulcan_gb300 import _build, capi
    _build.build()
    return capi.lib()


def header_symbols():
    src = open(os.path.join(REPO, 'include', 'vk_ros2.h')).read()
    return sorted(set(re.findall(r'VK_API\s+[\w\s\*]*?\b(vk_\w+)\s*\(', src)))


def test_exports_every_declared_symbol(lib):
    from vulcan_gb300 import capi
    names = header_symbols()
    assert len(names) >= 20
    assert sorted(capi.EXPORTS) == names
    for n in names:
        assert hasattr(lib, n), n


def test_no_closed_batch_copy_calls():
    """The library must not use the batched-memcpy family of calls."""
    pat = re.compile('Memcpy' + r'\w*Batch')
    for root, _, files in os.walk(os.path.join(REPO, 'vulcan_gb300', 'csrc')):
        for f in files:
            assert not pat.search(open(os.path.join(root, f)).read()), f


@pytest.mark.parametrize('tag', ['c0', 'c2'])
def test_network_tables_match_jacobian_structure(lib, tag):
    from vulcan_gb300.solver import GPUNetwork
    g = golden(tag)
    net = network(tag)
    gn = GPUNetwork(net, [str(a) for a in g['atom_list']])
    rows, cols = gn.jac_pattern()
    # structural pattern of the chemistry Jacobian from the oracle with all y = 1
    on = oracle_net(tag, g)
    ones = np.ones((1, net.ni))
    J = O.neg_jac_blocks(on, ones, np.ones(1), np.ones((net.nr, 1)))[0]
    ref = set(zip(*np.nonzero(J)))
    got = set(zip(rows.tolist(), cols.tolist()))
    assert ref <= got                     # every structural non-zero is stored
    assert len(got) == gn.nnz
    assert gn.nsrc >= 2 * net.npair - 2


def test_bad_descriptor_rejected(lib):
    from vulcan_gb300 import capi
    ptr = capi.ptr
    a = lambda v: np.ascontiguousarray(v, dtype=np.int32)
    rp, rs, rn = a([0, 2]), a([0, 99]), a([1, 1])   # species 99 out of range
    pp, ps, pn = a([0, 1]), a([1]), a([1])
    comp = np.zeros(2)
    d = capi.VkNetworkDesc(2, 1, ptr(rp, C.c_int), ptr(rs, C.c_int), ptr(rn, C.c_int),
                           ptr(pp, C.c_int), ptr(ps, C.c_int), ptr(pn, C.c_int), 1, ptr(comp))
    h = C.c_void_p()
    rc = lib.vk_network_compile(C.byref(d), C.byref(h))
    assert rc == capi.VK_EINVAL
    assert b'bad term' in lib.vk_network_last_error()
    assert not h.value


def test_null_handle_errors(lib):
    from vulcan_gb300 import capi
    assert lib.vk_set_columns(None, 1, None, None, None, None, None, None, None) == capi.VK_EINVAL
    assert lib.vk_last_error(None)


NO_HANDLE = ('vk_network_compile', 'vk_network_free', 'vk_network_last_error', 'vk_destroy',
             'vk_last_error', 'vk_group_destroy')


def test_every_entry_point_rejects_null_arguments(lib):
    """Each status-returning entry point answers VK_EINVAL to a NULL handle
    (zero sizes for the handle-free ones) before touching the device."""
    from vulcan_gb300 import capi
    checked = 0
    for name in capi.EXPORTS:
        if name in NO_HANDLE:
            continue
        f = getattr(lib, name)
        args = []
        for t in f.argtypes:
            if t in (C.c_int, C.c_longlong):
                args.append(0)
            elif t in (C.c_double, C.c_float):
                args.append(0.0)
            else:
                args.append(None)
        assert f(*args) == capi.VK_EINVAL, name
        checked += 1
    assert checked == len(capi.EXPORTS) - len(NO_HANDLE)


def test_group_arguments_checked_on_host(lib):
    """vk_group_create rejects an empty list, NULL and repeated handles
    before it creates any device object (the pointers are only compared)."""
    from vulcan_gb300 import capi
    out = C.c_void_p(1)
    fake = C.c_void_p(0x1000)
    arr = (C.c_void_p * 2)(fake, fake)
    assert lib.vk_group_create(arr, 0, C.byref(out)) == capi.VK_EINVAL
    assert out.value is None
    assert lib.vk_group_create(arr, 2, C.byref(out)) == capi.VK_EINVAL
    assert b'twice' in lib.vk_last_error(None)
    arr0 = (C.c_void_p * 2)(fake, None)
    assert lib.vk_group_create(arr0, 2, C.byref(out)) == capi.VK_EINVAL
    assert b'NULL' in lib.vk_last_error(None)
    assert lib.vk_group_create(arr, 1, None) == capi.VK_EINVAL
    lib.vk_group_destroy(None)


def test_c_client_builds_and_runs(lib, tmp_path):
    """A plain C program compiled against include/vk_ros2.h and linked to
    the library: network compile, table sizes, Jacobian pattern, error paths."""
    import shutil
    import subprocess
    from vulcan_gb300 import capi
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    libdir = os.path.dirname(capi.LIB)
    exe = str(tmp_path / 'c_abi_client')
    subprocess.run([cc, '-std=c99', '-Wall', '-Werror', '-I', os.path.join(REPO, 'include'),
                    os.path.join(REPO, 'tests', 'c_abi_client.c'), '-o', exe,
                    '-L', libdir, '-lvk_gb300', '-Wl,-rpath,' + libdir], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith('c-abi ok')
