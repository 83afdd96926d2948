"""The C ABI library loads and exports every function include/ declares;
host-only entry points (model compiler, options, statuses) work without a
GPU."""
import ctypes as C
import os
import re

import numpy as np

from lassie_gb300 import _native as nat
from lassie_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"\b(lassie_\w+)\s*\(", text))
    return names


def test_exports_every_declared_symbol(native):
    decl = declared_functions()
    assert decl, "no declarations found"
    assert decl <= set(nat.EXPORTS), decl - set(nat.EXPORTS)
    for name in decl:
        assert hasattr(native, name), name


def test_defaults_match_reference(native):
    o = nat.Opts()
    native.lassie_opts_default(C.byref(o))
    assert (o.rkf_step, o.be_step, o.newton_tol, o.stiffness_tol, o.newton_iter) == \
        (1e-3, 0.01, 1e-6, 1e-6, 10000)


def test_model_compiler_counts(native):
    m = synth.make_c1()
    left = np.ascontiguousarray(m.left, np.int32)
    right = np.ascontiguousarray(m.right, np.int32)
    h = C.c_void_p()
    assert native.lassie_model_create_dense(64, 64, left.ctypes.data, right.ctypes.data,
                                            C.byref(h)) == 0
    v = [C.c_int32() for _ in range(4)]
    assert native.lassie_model_info(h, *[C.byref(x) for x in v]) == 0
    assert [x.value for x in v] == [64, 64, int(np.count_nonzero(left)),
                                    int(np.count_nonzero(right - left))]
    native.lassie_model_destroy(h)


def test_csr_and_dense_agree(native):
    # A + B -> C, 2C -> A (given as CSR by reaction)
    rp = np.array([0, 2, 3], np.int32); rs = np.array([0, 1, 2], np.int32)
    rc = np.array([1, 1, 2], np.int32)
    pp = np.array([0, 1, 2], np.int32); ps = np.array([2, 0], np.int32)
    pc = np.array([1, 1], np.int32)
    h = C.c_void_p()
    assert native.lassie_model_create_csr(3, 2, rp.ctypes.data, rs.ctypes.data, rc.ctypes.data,
                                          pp.ctypes.data, ps.ctypes.data, pc.ctypes.data,
                                          C.byref(h)) == 0
    v = [C.c_int32() for _ in range(4)]
    native.lassie_model_info(h, *[C.byref(x) for x in v])
    assert [x.value for x in v] == [3, 2, 3, 5]
    native.lassie_model_destroy(h)


def test_bad_arguments_are_rejected(native):
    h = C.c_void_p()
    assert native.lassie_model_create_dense(0, 1, None, None, C.byref(h)) == nat.ERR_ARGS
    assert native.lassie_status_string(nat.ERR_MAX_STEPS) == b"maximum number of steps reached"
    # stoichiometry outside int8 is refused, not truncated
    left = np.array([[300]], np.int32); right = np.zeros((1, 1), np.int32)
    assert native.lassie_model_create_dense(1, 1, left.ctypes.data, right.ctypes.data,
                                            C.byref(h)) == nat.ERR_TOO_LARGE


def test_bdf_controller_options_checked_on_host(native):
    """BDF controller: defaults, and option / instance checks that run before
    any device query (so they hold without a GPU)."""
    from lassie_gb300 import solver
    o = nat.Opts()
    native.lassie_opts_default(C.byref(o))
    assert (o.controller, o.rtol, o.atol, o.max_order) == (nat.CTRL_COMPAT, 1e-6, 1e-9, 5)
    assert native.lassie_status_string(nat.ERR_STEP_TOO_SMALL).startswith(b"BDF step size")

    def create(m, **bdf):
        nm = solver.NativeModel.of(m)
        pk = solver._Packed(m, nm)
        inst = nat.Instance()
        inst.model, inst.k, inst.x0 = nm.handle, pk.k.ctypes.data, pk.x0.ctypes.data
        inst.t, inst.nt = pk.t.ctypes.data, pk.t.shape[0]
        inst.out, inst.cs, inst.ncs = pk.out.ctypes.data, None, 0
        opts = solver.make_opts(m, bdf=bdf)
        h = C.c_void_p()
        rc = native.lassie_batch_create(C.byref(inst), 1, C.byref(opts), C.byref(h))
        if rc == 0:
            native.lassie_batch_destroy(h)
        return rc

    m = synth.make_c1()
    assert create(m, rtol=0.0) == nat.ERR_ARGS
    assert create(m, max_order=6) == nat.ERR_ARGS
    assert create(m, max_step=-1.0) == nat.ERR_ARGS
    bad_t = synth.make_c1()
    bad_t.t = bad_t.t[::-1].copy()
    assert create(bad_t) == nat.ERR_ARGS          # sample times must ascend
    assert create(synth.make_sized(600, 0)) == nat.ERR_TOO_LARGE
    # valid options: the next check is the device (none here, or one on a GPU machine)
    assert create(m) in (nat.OK, nat.ERR_NO_DEVICE)


def test_jacobian_pattern_on_host(native):
    """lassie_jacobian_pattern / _nnz (host only): the structural nonzeros of
    J, columns ascending per row, equal to the nonzeros of the oracle's
    Jacobian at positive states (no cancellation at random x)."""
    from lassie_gb300 import solver
    from oracle import oracle as O
    for m in (synth.make_c1(), synth.make_c5(1)[0][0], synth.make_sized(77, 2),
              synth.tiny_network("reversible")):
        nm = solver.NativeModel.of(m)
        N = m.n_species
        nnz = C.c_int64()
        assert native.lassie_jacobian_nnz(nm.handle, C.byref(nnz)) == 0
        ptr = np.zeros(N + 1, np.int32)
        cols = np.zeros(max(1, nnz.value), np.int32)
        assert native.lassie_jacobian_pattern(nm.handle, ptr.ctypes.data, cols.ctypes.data) == 0
        assert ptr[-1] == nnz.value
        pat = np.zeros((N, N), bool)
        for i in range(N):
            row = cols[ptr[i]:ptr[i + 1]]
            assert np.all(np.diff(row) > 0)
            pat[i, row] = True
        om = O.OracleModel(m.left, m.right)
        rng = np.random.default_rng(N)
        seen = np.zeros((N, N), bool)
        for _ in range(3):
            seen |= om.jacobian(m.k, rng.uniform(0.1, 2.0, N)) != 0
        assert np.array_equal(seen, pat)


def test_adjoint_refuses_the_bdf_controller(native):
    """The adjoint differentiates LASSIE's loop; BDF options are refused on
    the host before any device work."""
    from lassie_gb300 import solver
    m = synth.make_c1()
    nm = solver.NativeModel.of(m)
    pk = solver._Packed(m, nm)
    inst = nat.Instance()
    inst.model, inst.k, inst.x0 = nm.handle, pk.k.ctypes.data, pk.x0.ctypes.data
    inst.t, inst.nt = pk.t.ctypes.data, pk.t.shape[0]
    inst.out, inst.cs, inst.ncs = pk.out.ctypes.data, None, 0
    target = np.zeros_like(pk.out)
    tp = (C.c_void_p * 1)(target.ctypes.data)
    g = np.zeros(m.n_reactions)
    gp = (C.c_void_p * 1)(g.ctypes.data)
    loss = np.zeros(1)
    opts = solver.make_opts(m, bdf={})
    rc = native.lassie_adjoint_batch(C.byref(inst), 1, C.cast(tp, C.c_void_p), C.byref(opts), 0, 0,
                                     loss.ctypes.data, C.cast(gp, C.c_void_p), None, None)
    assert rc == nat.ERR_ARGS


def test_tile_rows_option_checked_on_host(native):
    """lassie_opts.tile_rows: 0 (autotuned) by default; 8, 4 or 2 fix the
    factorisation's tile rows; anything else is refused before any device
    query."""
    from lassie_gb300 import solver
    o = nat.Opts()
    native.lassie_opts_default(C.byref(o))
    assert o.tile_rows == 0
    m = synth.make_c1()
    nm = solver.NativeModel.of(m)
    pk = solver._Packed(m, nm)
    inst = nat.Instance()
    inst.model, inst.k, inst.x0 = nm.handle, pk.k.ctypes.data, pk.x0.ctypes.data
    inst.t, inst.nt = pk.t.ctypes.data, pk.t.shape[0]
    inst.out, inst.cs, inst.ncs = pk.out.ctypes.data, None, 0
    for rows, want in ((3, (nat.ERR_ARGS,)), (16, (nat.ERR_ARGS,)), (-1, (nat.ERR_ARGS,)),
                       (4, (nat.OK, nat.ERR_NO_DEVICE))):
        opts = solver.make_opts(m, tile_rows=rows)
        h = C.c_void_p()
        rc = native.lassie_batch_create(C.byref(inst), 1, C.byref(opts), C.byref(h))
        if rc == 0:
            native.lassie_batch_destroy(h)
        assert rc in want, (rows, rc)
