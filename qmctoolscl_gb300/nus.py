"""Nested uniform (Owen) scrambling of base-2 digital nets on the GPU:
``dnb2_nested_uniform_scramble`` with the reference's arguments and results
(qmctoolscl/rand_funcs.py:155-253), bit for bit, numpy generator streams
included.

The reference walks a binary tree per (replication, dimension), point by
point, drawing fresh random bits from that pair's numpy Generator whenever a
point opens a new branch.  The result is fixed by three facts, which the GPU
computes in parallel instead of walking the tree:

* the root is a leaf for a phantom point 0 that holds tmax_new random bits,
  drawn first;
* point v draws tmax_new - L_v - 1 bits (none when the point repeats an
  earlier one), where L_v is the longest common prefix (in tmax_new-bit keys,
  xb << (tmax_new - tmax)) between v and any earlier point -- the draws come
  from the generator in point order, so one pass per generator assigns them;
* the bit of the scramble at depth k of a point comes from the draw of the
  earliest point that shares the point's first k bits.

The kernels sort each generator's keys, build a binary radix tree over them,
take each subtree's earliest point bottom-up (which gives every L_v), run the
draws (one thread per generator, numpy's SFC64 stream and bounded-integer
rule), and OR each point's bits from its ancestors' draws.

Generators must be ``numpy.random.Generator(numpy.random.SFC64(...))`` (the
reference's own family), one per (l, j) pair, as the reference's documented
use spawns them; their states are read before the call and set to the
advanced states after it, so later draws continue exactly as after the
reference's call.  One generator serving several pairs is refused
(ValueError): the reference would draw its stream across those pairs in
turn, which the per-pair parallel passes do not reproduce.  Root nodes are ``NUSNode_dnb2`` objects of this module: a
fresh node starts a tree; a node used by an earlier call keeps that call's
points and draws, so a later call extends the same scramble as the reference
does with its own nodes.
"""
import ctypes
import time

import numpy as np

from . import _ffi

STATE_WORDS = 6  # a, b, c, w, has_uint32, uinteger


def sfc64_state_words(rng):
    """The six state words (a, b, c, w, has_uint32, uinteger) of a numpy
    Generator on an SFC64 bit generator."""
    bg = getattr(rng, "bit_generator", None)
    st = bg.state if bg is not None else None
    if st is None or st.get("bit_generator") != "SFC64":
        raise TypeError("nested uniform scrambling needs numpy.random.Generator(numpy.random.SFC64(...)) "
                        "generators, got %r" % (rng,))
    w = np.zeros(STATE_WORDS, dtype=np.uint64)
    w[:4] = np.asarray(st["state"]["state"], dtype=np.uint64)
    w[4] = int(st["has_uint32"])
    w[5] = int(st["uinteger"])
    return w


def set_sfc64_state(rng, words):
    """Set a Generator's SFC64 state from six words (the inverse of sfc64_state_words)."""
    bg = rng.bit_generator
    st = bg.state
    st["state"]["state"] = np.asarray(words[:4], dtype=np.uint64).copy()
    st["has_uint32"] = int(words[4])
    st["uinteger"] = int(words[5])
    bg.state = st


class NUSNode_dnb2(object):
    """Root of one generator's scrambling tree, with the fields of the
    reference's node (qmctoolscl/rand_funcs.py:155-160).  A fresh node
    (shift_bits None) starts a tree.  After a call, shift_bits holds the
    root's tmax_new random bits and the node keeps the tree's history on the
    GPU: the keys and draws of every entry the tree has seen, which a later
    call on the same node continues from."""

    def __init__(self, shift_bits=None, xb=None, left_b2=None, right_b2=None):
        self.shift_bits = shift_bits
        self.xb = xb
        self.left_b2 = left_b2
        self.right_b2 = right_b2
        self._hist = None  # (keys, draws, tmax_new): device rows of one generator


def _t():
    import torch
    return torch


def _objects(a, r, d, what):
    arr = np.empty(r * d, dtype=object)
    flat = list(np.asarray(a, dtype=object).reshape(-1))
    if len(flat) != r * d:
        raise ValueError("%s holds %d entries, the call needs r*d = %d" % (what, len(flat), r * d))
    arr[:] = flat
    return arr


def _u64_array(a, need, name, pos):
    """(device tensor, numpy array or None) for a uint64 argument."""
    torch = _t()
    if type(a).__module__.startswith("torch"):
        if a.dtype not in (torch.int64, torch.uint64) or not a.is_cuda or not a.is_contiguous():
            raise ctypes.ArgumentError("argument %d (%s): contiguous CUDA int64/uint64 tensor required" % (pos, name))
        if a.numel() < need:
            raise ValueError("%s has %d elements, the call needs %d" % (name, a.numel(), need))
        return a, None
    if not isinstance(a, np.ndarray) or a.dtype != np.uint64 or not a.flags["C_CONTIGUOUS"]:
        raise ctypes.ArgumentError("argument %d (%s): C-contiguous numpy uint64 array required" % (pos, name))
    if a.size < need:
        raise ValueError("%s has %d elements, the call needs %d" % (name, a.size, need))
    return None, a


_ATTRS = {}


def _host_writable(arr, allowed):
    """Address at which the kernels may write the numpy array `arr` directly, or
    None: the device alias of pinned memory, or the array's own address where
    the GPU reaches pageable host memory through the host's page tables (GB300
    next to a Grace CPU).  Otherwise the result goes through a device buffer
    and a copy."""
    if not allowed:
        return None
    ptr = arr.ctypes.data
    dev_ptr = _ffi.device_pointer_of_host(ptr)
    if dev_ptr is not None:
        return dev_ptr
    if "a" not in _ATTRS:
        _ATTRS["a"] = _ffi.device_attributes()
    a = _ATTRS["a"]
    if a["pageable_access"] and a["uses_host_page_tables"]:
        return ptr
    return None


def workspace_bytes(n, h0, generators):
    """Device bytes the kernels need to scramble `generators` generators at once."""
    lib = _ffi.lib()
    out = ctypes.c_uint64(0)
    _ffi.check(lib.qmc_dnb2_nus_workspace_size(n, h0, generators, ctypes.byref(out)), "dnb2_nested_uniform_scramble")
    return out.value


def dnb2_nested_uniform_scramble(r, n, d, r_x, tmax, tmax_new, rngs, root_nodes, xb, xrb, **kwargs):
    """Nested uniform scramble of digital net b2

Args:
    r (np.uint64): replications
    n (np.uint64): points
    d (np.uint64): dimensions
    r_x (np.uint64): replications of xb
    tmax (np.uint64): maximum number of bits in each integer
    tmax_new (np.uint64): maximum number of bits in each integer after scrambling
    rngs (np.ndarray of numpy.random._generator.Generator): random number generators of size r*d
    root_nodes (np.ndarray of NUSNode_dnb2): root nodes of size r*d
    xb (np.ndarray of np.uint64): array of unrandomized points of size r*n*d
    xrb (np.ndarray of np.uint64): array to store scrambled points of size r*n*d

Keyword arguments (beyond the reference): ``workspace_bytes`` caps the
device scratch (default: half the free device memory, at most 160 GiB, so that every
generator runs in one chunk with one serial draw pass where that fits);
generators run in chunks that fit it.  ``stream`` selects a
torch.cuda.Stream.  ``host_writes`` (default True): a numpy ``xrb`` is
written by the kernels directly where the GPU can reach it (pinned memory,
or pageable memory through the host's page tables), else copied back."""
    t0_perf = time.perf_counter()
    t0_process = time.process_time()
    torch = _t()
    r, n, d, r_x, tmax, tmax_new = (int(v) for v in (r, n, d, r_x, tmax, tmax_new))
    G = r * d
    gens = _objects(rngs, r, d, "rngs")
    roots = _objects(root_nodes, r, d, "root_nodes")
    for node in roots:
        assert isinstance(node, NUSNode_dnb2)
    fresh = [node.shift_bits is None for node in roots]
    if all(fresh):
        h0 = 0
        assert 0 <= tmax_new <= 64, "t must be between 0 and 64"
    elif not any(fresh) and all(node._hist is not None for node in roots):
        h0s = {int(node._hist[0].numel()) for node in roots}
        if len(h0s) != 1:
            raise ValueError("root_nodes hold trees of different sizes; scramble them in separate calls")
        h0 = h0s.pop()
        if any(node._hist[2] != tmax_new for node in roots):
            raise ValueError("root_nodes were built with another tmax_new")
    else:
        raise ValueError("root_nodes must be all fresh or all built by earlier calls of this function")
    if len({id(getattr(g, "bit_generator", g)) for g in gens}) != G:
        raise ValueError("rngs must hold r*d distinct generators: the reference draws a shared generator's "
                         "stream across the (l, j) pairs it serves, one pair after another")
    dxb, hxb = _u64_array(xb, r_x * n * d, "xb", 9)
    dxrb, hxrb = _u64_array(xrb, r * n * d, "xrb", 10)
    states = np.stack([sfc64_state_words(g) for g in gens]) if G else np.zeros((0, STATE_WORDS), np.uint64)
    lib = _ffi.lib()
    dev = dxb.device if dxb is not None else (dxrb.device if dxrb is not None else
                                              torch.device("cuda", torch.cuda.current_device()))
    stream = kwargs.get("stream") or torch.cuda.current_stream(dev)
    if G == 0:
        return time.perf_counter() - t0_perf, time.process_time() - t0_process
    H = (h0 if h0 else 1) + n
    per = workspace_bytes(n, h0, 1)
    budget = kwargs.get("workspace_bytes")
    if budget is None:
        free, _total = torch.cuda.mem_get_info(dev)
        budget = min(free // 2, 160 << 30)  # one chunk, one serial draw pass, where it fits
    count = max(1, min(G, int(budget) // per))
    wbytes = workspace_bytes(n, h0, count)
    with torch.cuda.device(dev), torch.cuda.stream(stream):
        i64 = torch.int64
        dstate = torch.from_numpy(states.reshape(-1).view(np.int64)).to(dev)
        if dxb is None:
            dxb = torch.from_numpy(_ffi.writable(hxb.reshape(-1)[:r_x * n * d].view(np.int64))).to(dev) if n else \
                torch.empty(1, dtype=i64, device=dev)
        xrb_ptr = None
        if dxrb is None and n:
            xrb_ptr = _host_writable(hxrb, kwargs.get("host_writes", True))
        if dxrb is None and xrb_ptr is None:
            dxrb = torch.empty(max(r * n * d, 1), dtype=i64, device=dev)
        if xrb_ptr is None:
            xrb_ptr = dxrb.data_ptr()
        if h0:
            hk = torch.stack([node._hist[0] for node in roots]).contiguous()
            hd = torch.stack([node._hist[1] for node in roots]).contiguous()
        else:
            hk = hd = None
        keys_out = torch.empty((G, H), dtype=i64, device=dev)
        draws_out = torch.empty((G, H), dtype=i64, device=dev)
        work = torch.empty(wbytes, dtype=torch.uint8, device=dev)
        rc = lib.qmc_dnb2_nested_uniform_scramble(
            r, n, d, r_x, tmax, tmax_new, dstate.data_ptr(), h0, hk.data_ptr() if h0 else None,
            hd.data_ptr() if h0 else None, dxb.data_ptr(), xrb_ptr, keys_out.data_ptr(),
            draws_out.data_ptr(), work.data_ptr(), wbytes, stream.cuda_stream)
        _ffi.check(rc, "dnb2_nested_uniform_scramble")
        if hxrb is not None and n and dxrb is not None:
            torch.from_numpy(hxrb.reshape(-1)[:r * n * d].view(np.int64)).copy_(dxrb[:r * n * d])
        new_states = dstate.cpu().numpy().view(np.uint64).reshape(G, STATE_WORDS)
        roots_bits = draws_out[:, 0].cpu().numpy().view(np.uint64)
        _ffi.check(lib.qmc_device_error_check(stream.cuda_stream), "dnb2_nested_uniform_scramble")
        del work
    for k in range(G):
        set_sfc64_state(gens[k], new_states[k])
        node = roots[k]
        node.shift_bits = np.uint64(roots_bits[k])
        node._hist = (keys_out[k], draws_out[k], tmax_new)
    return time.perf_counter() - t0_perf, time.process_time() - t0_process


class NUSNode_gdn(object):
    """Root of one generator's base-b scrambling tree, with the fields of the
    reference's node (qmctoolscl/rand_funcs.py:255-260).  A fresh node (perm
    None) starts a tree.  After a call the node is marked used (perm set) and
    keeps its tree on the GPU: the keys of every entry so far (the phantom
    root and every point, in call order) and the permutation rows they drew,
    which a later call on the same node continues from."""

    def __init__(self, perm=None, xdig=None, children=None):
        self.perm = perm
        self.xdig = xdig
        self.children = children


def gdn_workspace_bytes(n, h0, generators):
    """Device bytes the kernels need to scramble `generators` base-b generators
    at once, n new points on trees of h0 entries so far (0: fresh trees)."""
    lib = _ffi.lib()
    out = ctypes.c_uint64(0)
    _ffi.check(lib.qmc_gdn_nus_workspace_size(n, h0, generators, ctypes.byref(out)), "gdn_nested_uniform_scramble")
    return out.value


def _perm_guess(n, h0_entries, tmax_new, base_of):
    """A first guess at the permutation entries all trees need: every point
    below the digits n points share draws the remaining levels (exact sizes
    come back from the call when the guess is short)."""
    total = h0_entries
    for b in base_of:
        share = int(np.floor(np.log(max(n, 1)) / np.log(b) + 1e-9))
        total += (n + 1) * b * max(1, tmax_new - share + 1)
    return total


def gdn_nested_uniform_scramble(r, n, d, r_x, r_b, tmax, tmax_new, rngs, root_nodes, bases, xdig, xrdig, **kwargs):
    """Nested uniform scramble of general digital nets

Args:
    r (np.uint64): replications
    n (np.uint64): points
    d (np.uint64): dimensions
    r_x (np.uint64): replications of xb
    r_b (np.uint64): replications of bases
    tmax (np.uint64): maximum number digits in each point representation
    tmax_new (np.uint64): maximum number digits in each point representation after scrambling
    rngs (np.ndarray of numpy.random._generator.Generator): random number generators of size r*d
    root_nodes (np.ndarray of NUSNode_gdn): root nodes of size r*d
    bases (np.ndarray of np.uint64): array of bases of size r*d
    xdig (np.ndarray of np.uint64): array of unrandomized points of size r*n*d*tmax
    xrdig (np.ndarray of np.uint64): array to store scrambled points of size r*n*d*tmax_new

Runs on the GPU with bases 2..65536, tmax < tmax_new <= 255 and
tmax * ceil(log2 b) <= 128 (ValueError otherwise).  A digit at or above its
base raises IndexError, as the reference does.  A later call on the same
root nodes continues their trees as the reference's nodes do: each node
keeps, on the GPU, the keys of every point its tree has seen (16 bytes each)
and the permutations they drew (2 bytes per entry, b entries per level), and
new points draw from the generators' current states.  Keyword arguments:
``workspace_bytes`` caps the device scratch, ``stream`` selects a
torch.cuda.Stream."""
    t0_perf = time.perf_counter()
    t0_process = time.process_time()
    torch = _t()
    r, n, d, r_x, r_b, tmax, tmax_new = (int(v) for v in (r, n, d, r_x, r_b, tmax, tmax_new))
    G = r * d
    gens = _objects(rngs, r, d, "rngs")
    roots = _objects(root_nodes, r, d, "root_nodes")
    for node in roots:
        assert isinstance(node, NUSNode_gdn)
    if len({id(getattr(g, "bit_generator", g)) for g in gens}) != G:
        raise ValueError("rngs must hold r*d distinct generators: the reference draws a shared generator's "
                         "stream across the (l, j) pairs it serves, one pair after another")
    bases_np = np.ascontiguousarray(np.asarray(bases, dtype=np.uint64)).reshape(-1)
    if bases_np.size < r_b * d:
        raise ValueError("bases has %d elements, the call needs r_b*d = %d" % (bases_np.size, r_b * d))
    bases_np = bases_np[:r_b * d]
    if G and (bases_np.min() < 2 or bases_np.max() > 65536):
        raise ValueError("bases must lie in 2..65536 for the GPU form")
    if not (1 <= tmax < tmax_new <= 255):
        raise ValueError("the GPU form needs 1 <= tmax < tmax_new <= 255 (tmax=%d, tmax_new=%d)" % (tmax, tmax_new))
    if G and tmax * int(np.ceil(np.log2(float(bases_np.max())))) > 128:
        raise ValueError("tmax * ceil(log2 b) must not exceed 128 bits for the GPU form")
    dxd, hxd = _u64_array(xdig, r_x * n * d * tmax, "xdig", 11)
    dxr, hxr = _u64_array(xrdig, r * n * d * tmax_new, "xrdig", 12)
    base_of = [int(bases_np[(k // d % r_b) * d + k % d]) for k in range(G)]
    fresh = [node.perm is None for node in roots]
    h0 = 0
    if all(fresh):
        pass
    elif not any(fresh) and all(getattr(node, "_hist", None) is not None for node in roots):
        hs = {int(node._hist["keys"].shape[0]) for node in roots}
        if len(hs) != 1:
            raise ValueError("root_nodes hold trees of different sizes; scramble them in separate calls")
        h0 = hs.pop()
        for k, node in enumerate(roots):
            hk = node._hist
            if (hk["tmax"], hk["tmax_new"], hk["base"]) != (tmax, tmax_new, base_of[k]):
                raise ValueError("root_nodes were built with another tmax, tmax_new or base")
    else:
        raise ValueError("root_nodes must be all fresh or all built by earlier calls of this function")
    if G == 0:
        return time.perf_counter() - t0_perf, time.process_time() - t0_process
    states = np.stack([sfc64_state_words(g) for g in gens])
    lib = _ffi.lib()
    dev = dxd.device if dxd is not None else (dxr.device if dxr is not None else
                                              torch.device("cuda", torch.cuda.current_device()))
    stream = kwargs.get("stream") or torch.cuda.current_stream(dev)
    H0 = h0 if h0 else 1
    N = H0 + n
    per = gdn_workspace_bytes(n, h0, 1)
    budget = kwargs.get("workspace_bytes")
    if budget is None:
        free, _total = torch.cuda.mem_get_info(dev)
        budget = min(free // 4, 32 << 30)
    count = max(1, min(G, int(budget) // per))
    wbytes = gdn_workspace_bytes(n, h0, count)
    with torch.cuda.device(dev), torch.cuda.stream(stream):
        i64 = torch.int64
        dbases = torch.from_numpy(bases_np.view(np.int64)).to(dev)
        if dxd is None:
            dxd = torch.from_numpy(_ffi.writable(hxd.reshape(-1)[:r_x * n * d * tmax].view(np.int64))).to(dev) \
                if n else torch.empty(1, dtype=i64, device=dev)
        if dxr is None:
            dxr = torch.empty(max(r * n * d * tmax_new, 1), dtype=i64, device=dev)
        if h0:
            hist_keys = torch.stack([node._hist["keys"] for node in roots]).contiguous()
            hist_rows = torch.cat([node._hist["perms"] for node in roots]) if G else None
            lens = np.array([int(node._hist["perms"].numel()) for node in roots], dtype=np.int64)
            hist_off = torch.from_numpy(np.concatenate([[0], np.cumsum(lens)])).to(dev)
            old_entries = int(lens.sum())
        else:
            hist_keys = hist_rows = hist_off = None
            old_entries = 0
        keys_out = torch.empty((G, N, 2), dtype=i64, device=dev)
        work = torch.empty(wbytes, dtype=torch.uint8, device=dev)
        capacity = _perm_guess(n, old_entries, tmax_new, base_of)
        needed = ctypes.c_uint64(0)
        perm_off = np.zeros(G + 1, dtype=np.uint64)
        for _attempt in range(2):
            dstate = torch.from_numpy(states.reshape(-1).view(np.int64)).to(dev)
            perms = torch.empty(max(capacity, 1), dtype=torch.int16, device=dev)
            rc = lib.qmc_gdn_nested_uniform_scramble(
                r, n, d, r_x, r_b, tmax, tmax_new, dstate.data_ptr(), dbases.data_ptr(), h0,
                hist_keys.data_ptr() if h0 else None, hist_rows.data_ptr() if h0 else None,
                hist_off.data_ptr() if h0 else None, dxd.data_ptr(), dxr.data_ptr(), keys_out.data_ptr(),
                perms.data_ptr(), capacity, perm_off.ctypes.data, ctypes.byref(needed), work.data_ptr(), wbytes,
                stream.cuda_stream)
            if rc == _ffi.QMC_ERR_ARG and needed.value > capacity:
                del perms
                capacity = int(needed.value)
                continue
            _ffi.check(rc, "gdn_nested_uniform_scramble")
            break
        else:
            raise _ffi.QmcError("gdn_nested_uniform_scramble: permutation buffer sizing did not settle")
        rc = lib.qmc_device_error_check(stream.cuda_stream)
        if rc == _ffi.QMC_ERR_DEVICE:
            raise IndexError("gdn_nested_uniform_scramble: a digit at or above its base")
        _ffi.check(rc, "gdn_nested_uniform_scramble")
        if hxr is not None and n:
            torch.from_numpy(hxr.reshape(-1)[:r * n * d * tmax_new].view(np.int64)).copy_(dxr[:r * n * d * tmax_new])
        new_states = dstate.cpu().numpy().view(np.uint64).reshape(G, STATE_WORDS)
        del work, hist_keys, hist_rows, hist_off
    for k in range(G):
        set_sfc64_state(gens[k], new_states[k])
        roots[k].perm = np.zeros(0, dtype=np.uint64)  # used; the tree lives in _hist
        roots[k]._hist = {"keys": keys_out[k], "perms": perms[int(perm_off[k]):int(perm_off[k + 1])],
                          "tmax": tmax, "tmax_new": tmax_new, "base": base_of[k]}
    return time.perf_counter() - t0_perf, time.process_time() - t0_process
