"""NumPy restatement of a tiled mesh's boundary exchange (both bc_vars) and
of fixup::FixFluxes.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker.  The product
never loads it.

The exchange follows the reference's sequence literally, block by block, on
host Blocks (numpy arrays shaped (nvar, k, j, i)):

1. neighbour exchange (Parthenon's AddBoundaryExchangeTasks,
   phoebus_driver.cpp:646-653): a ghost whose global cell -- after periodic
   wraps -- lies inside the domain receives the owning block's primitives
   and conserved variables (both carry FillGhost under bc_vars = primitive,
   fluid.cpp:153-165).  Ghosts beyond a physical face are left as they are;
   this restatement sets them to NaN first, so that any value the later
   steps fail to overwrite shows up.
2. ApplyBoundaryConditions: the block's physical faces in the order inner_x1,
   outer_x1, inner_x2, outer_x2, inner_x3, outer_x3, each over its ghost slab
   spanning the entire range of the other two axes, on every FillGhost
   variable (scaled by robust::ratio(DetGamma(ghost), DetGamma(source)) when
   bc_vars = conserved): gr_outflow copies the boundary cell (OutflowInnerX1,
   OutflowOuterX1 phoebus_boundaries.cpp:115-150, 215-254; GenericBC Outflow
   :42-113), reflect copies the mirror cell with the components of vector
   variables along the axis negated (GenericBC Reflect), polar copies the
   mirror cell with v^2 and B^2 negated (PolarInnerX2, PolarOuterX2
   :153-213).
3. ConvertBoundaryConditions (:303-472): on an FMKS mesh with
   enable_ox1_fmks_inflow_check, u^1 >= 0 is enforced in the outer-X1 slab of
   a block on the outer X1 boundary (:366-397) and the slab is prim2con'd
   (:416); with bc_vars = conserved the slab goes through con2prim first
   (ConservedToPrimitiveRegion, :333-340).  With bc_vars = primitive, prim2con
   then runs over every physical slab (PrimitiveToConservedRegion, through
   the C oracle).

FixFluxes follows fixup.cpp:728-1078 on the blocks' flux arrays.
"""
from __future__ import annotations

import numpy as np

from phoebus_gb300 import abi

PERIODIC, OUTFLOW, REFLECT, POLAR = abi.BC_PERIODIC, abi.BC_OUTFLOW, abi.BC_REFLECT, abi.BC_POLAR
# conserved layout: D, S_1..3, tau, B^1..3
CRHO, CMOM, CENG, CB = 0, 1, 4, 5


def _origin(mesh, seg):
    return tuple(int(mesh.starts[d][seg[d]]) for d in range(3))


def _owner_cell(mesh, g):
    """(block index, local interior index per axis) of global cell g."""
    s = tuple(int(np.searchsorted(mesh.starts[d], g[d], side="right") - 1) for d in range(3))
    return mesh.block_index(*s), tuple(g[d] - int(mesh.starts[d][s[d]]) for d in range(3))


def _pvars(mhd):
    """The primitive variables present (no B without MHD)."""
    return [v for v in range(abi.NPRIM) if mhd or not (abi.PB <= v < abi.PB + 3)]


def _exchange_neighbours(mesh, blocks, mhd):
    ncons = abi.NCONS if mhd else 5
    pv = _pvars(mhd) if mesh.bc_vars == abi.BC_VARS_PRIMITIVE else []
    _copy_neighbours(mesh, blocks, [("prim", pv), ("cons", range(ncons))])


def _copy_neighbours(mesh, blocks, fields):
    """Parthenon's exchange of the FillGhost fields: fields = [(array name,
    variable indices)]."""
    segs = list(mesh.segments())
    src = [{n: b[n].copy() for n, _ in fields} for b in blocks]  # owners' values before this exchange
    for b, seg in zip(blocks, segs):
        ng = b.ng
        org = _origin(mesh, seg)
        shape_t = (b.n1t, b.n2t, b.n3t)
        gg, inside, interior, owner_seg, local = [], [], [], [], []
        for d in range(3):
            if d >= b.ndim:  # inactive axis: one cell, no ghosts
                for lst, val in ((gg, [0]), (inside, [True]), (interior, [True]), (owner_seg, [0]), (local, [0])):
                    lst.append(np.array(val))
                continue
            loc = np.arange(shape_t[d])
            g = org[d] + loc - ng
            lo, hi = g < 0, g >= mesh.n[d]
            ins = np.ones_like(lo)
            if mesh.bc_lo[d] == PERIODIC:
                g = np.where(lo, g + mesh.n[d], g)
            else:
                ins &= ~lo
            if mesh.bc_hi[d] == PERIODIC:
                g = np.where(hi, g - mesh.n[d], g)
            else:
                ins &= ~hi
            gc = np.clip(g, 0, mesh.n[d] - 1)
            sg = np.searchsorted(mesh.starts[d], gc, side="right") - 1
            gg.append(gc)
            inside.append(ins)
            interior.append((loc >= ng) & (loc < ng + b.nx[d]))
            owner_seg.append(sg)
            local.append(gc - mesh.starts[d][sg] + ng)
        # (k, j, i) grids
        I, J, K = np.meshgrid(np.arange(b.n1t), np.arange(b.n2t), np.arange(b.n3t), indexing="ij")
        I, J, K = I.transpose(2, 1, 0), J.transpose(2, 1, 0), K.transpose(2, 1, 0)
        ghost = ~(interior[0][I] & interior[1][J] & interior[2][K])
        ins = inside[0][I] & inside[1][J] & inside[2][K]
        out = ghost & ~ins
        for n, vs in fields:
            for v in vs:
                b[n][v][out] = np.nan
        take = ghost & ins
        own = np.vectorize(mesh.block_index)(owner_seg[0][I], owner_seg[1][J], owner_seg[2][K])
        li, lj, lk = local[0][I], local[1][J], local[2][K]
        for o in np.unique(own[take]):
            m = take & (own == o)
            for n, vs in fields:
                for v in vs:
                    b[n][v][m] = src[o][n][v][lk[m], lj[m], li[m]]


def _physical_faces(mesh, b, seg):
    """[(axis, outer, bc)] of the block's faces on a physical boundary, in
    the order Parthenon applies them."""
    org = _origin(mesh, seg)
    out = []
    for d in range(b.ndim):
        for outer in (False, True):
            bc = mesh.bc_hi[d] if outer else mesh.bc_lo[d]
            edge = org[d] + b.nx[d] == mesh.n[d] if outer else org[d] == 0
            if edge and bc != PERIODIC:
                out.append((d, outer, bc))
    return out


def _detg(b):
    """DetGamma at cell centres, shaped (k, j, i) by broadcasting (1 in
    Minkowski)."""
    if b.geom is None:
        return np.ones((1, b.n2t, b.n1t))
    return b.geom.arrays["cent"][abi.G_DETGAM][None, :, :]


def _ratio(a, b):
    """robust::ratio (robust.hpp:35-39)."""
    small = 10 * np.finfo(np.float64).tiny
    return a / (b + np.where(b >= 0, 1.0, -1.0) * small)


def _apply_face(b, d, outer, bc, mhd, bc_vars):
    """One boundary function on one block (all FillGhost variables)."""
    ng, nd = b.ng, b.nx[d]
    lo_i, hi_i = ng, ng + nd - 1  # interior range on axis d (local)
    ghosts = range(hi_i + 1, hi_i + 1 + ng) if outer else range(0, ng)
    ref = hi_i if outer else lo_i
    axis = 3 - d  # array axis of dimension d in (var, k, j, i)
    P, U = b["prim"], b["cons"]
    ncons = abi.NCONS if mhd else 5
    conserved = bc_vars == abi.BC_VARS_CONSERVED
    pvars = [] if conserved else _pvars(mhd)
    detg = np.broadcast_to(_detg(b), (b.n3t, b.n2t, b.n1t))
    for g in ghosts:
        if bc == OUTFLOW:
            r = ref
        else:  # reflect / polar mirror: offset = 2 ref -/+ 1 (GenericBC), jref = -j + 2 j0 - 1 (polar)
            r = (2 * ref + (1 if outer else -1)) - g
        dst = [slice(None)] * 4
        src = [slice(None)] * 4
        dst[axis], src[axis] = g, r
        pv = P[tuple(src)].copy()
        uv = U[tuple(src)].copy()
        sp, su = np.ones(abi.NPRIM), np.ones(abi.NCONS)
        if bc == REFLECT:  # VectorComponent(l) == DIR: velocity, B (prims); S, B (cons)
            sp[abi.PVEL + d] = sp[abi.PB + d] = -1.0
            su[CMOM + d] = su[CB + d] = -1.0
        elif bc == POLAR:  # idx_pvel(1), idx_pb(1) only
            sp[abi.PVEL + 1] = sp[abi.PB + 1] = -1.0
        if conserved:  # q = sgn * gratio * q(ref)
            gratio = _ratio(detg[tuple(dst[1:])], detg[tuple(src[1:])])
            for v in range(ncons):
                U[(v,) + tuple(dst[1:])] = su[v] * gratio * uv[v]
        else:
            for v in pvars:
                P[(v,) + tuple(dst[1:])] = sp[v] * pv[v]
            for v in range(ncons):
                U[(v,) + tuple(dst[1:])] = su[v] * uv[v]


def _slab(b, d, outer):
    """(ib, jb, kb) inclusive ranges of a face's ghost slab, entire on the
    other axes (IndexDomain::inner_x1 & co.)."""
    r = list(b.entire())
    ng, nd = b.ng, b.nx[d]
    r[d] = (ng + nd, 2 * ng + nd - 1) if outer else (0, ng - 1)
    return tuple(r)


def _inflow_check(b, ib, jb, kb):
    """phoebus_boundaries.cpp:366-397 (fluid part): u^1 >= 0.  Elementwise
    over the slab, in the reference's operation order."""
    ks, js, is_ = slice(kb[0], kb[1] + 1), slice(jb[0], jb[1] + 1), slice(ib[0], ib[1] + 1)
    t = b.geom.arrays["cent"][:, js, is_][:, None, :, :]  # axisymmetric: broadcast over k
    P = b["prim"]
    gam = [[None] * 3 for _ in range(3)]
    for a in range(3):
        for c in range(3):
            hi, lo = max(a + 1, c + 1), min(a + 1, c + 1)
            gam[a][c] = t[abi.G_GCOV + hi * (hi + 1) // 2 + lo]
    alpha, beta0 = t[abi.G_ALPHA], t[abi.G_BETA]
    v = [P[abi.PVEL + a, ks, js, is_].copy() for a in range(3)]

    def vsq_of(v):
        s = np.zeros_like(v[0])
        for a in range(3):
            for c in range(3):
                s = s + gam[a][c] * v[a] * v[c]
        return s

    W = np.sqrt(1.0 + vsq_of(v))
    ucon1 = v[0] - W * beta0 / alpha
    fix = ucon1 < 0
    w = [x / W for x in v]
    w[0] = np.broadcast_to(beta0 / alpha, w[0].shape).copy()
    with np.errstate(invalid="ignore", divide="ignore"):  # cells that keep v may give NaN here
        W2 = 1.0 / np.sqrt(1.0 - vsq_of(w))
    for a in range(3):
        P[abi.PVEL + a, ks, js, is_] = np.where(fix, W2 * w[a], v[a])


def mesh_exchange(orc, p, mesh, blocks):
    """The whole exchange on host blocks, in place (orc: oracle.Oracle)."""
    mhd = bool(p.mhd)
    _exchange_neighbours(mesh, blocks, mhd)
    segs = list(mesh.segments())
    for b, seg in zip(blocks, segs):
        for d, outer, bc in _physical_faces(mesh, b, seg):
            _apply_face(b, d, outer, bc, mhd, mesh.bc_vars)
    conserved = mesh.bc_vars == abi.BC_VARS_CONSERVED
    for b, seg in zip(blocks, segs):
        faces = _physical_faces(mesh, b, seg)
        fmks = b.geom is not None
        if fmks and p.enable_ox1_fmks_inflow_check and any(d == 0 and outer for d, outer, _ in faces):
            ib, jb, kb = _slab(b, 0, True)
            if conserved:  # ConservedToPrimitiveRegion over the slab first (:333-340)
                orc.ConservedToPrimitive(p, b, ib, jb, kb)
            _inflow_check(b, ib, jb, kb)
            orc.PrimitiveToConserved(p, b, ib, jb, kb)
        if not conserved:
            for d, outer, _ in faces:
                orc.PrimitiveToConserved(p, b, *_slab(b, d, outer))


# ------------------------------------------------------------------ radiation
# The FillGhost radiation fields (radiation.cpp:448-474, 506-508): E, F_i and
# the primitives J, H_i/J, xi, phi, c2pfail (the first RFAIL + 1 of rprim).
RFILL = abi.RFAIL + 1


def _rad_apply_face(b, d, outer, bc, bc_vars):
    """One boundary function on the radiation fields of one block: every
    FillGhost field, scaled by the DetGamma ratio under bc_vars = conserved
    (GenericBC's rescale covers the radiation primitives too), F_d and H_d
    negated across a reflect face (Metadata::Vector); the polar functions
    negate only the fluid's v^2 and B^2."""
    ng, nd = b.ng, b.nx[d]
    lo_i, hi_i = ng, ng + nd - 1
    ghosts = range(hi_i + 1, hi_i + 1 + ng) if outer else range(0, ng)
    ref = hi_i if outer else lo_i
    axis = 3 - d
    conserved = bc_vars == abi.BC_VARS_CONSERVED
    detg = np.broadcast_to(_detg(b), (b.n3t, b.n2t, b.n1t))
    for g in ghosts:
        r = ref if bc == OUTFLOW else (2 * ref + (1 if outer else -1)) - g
        dst = [slice(None)] * 4
        src = [slice(None)] * 4
        dst[axis], src[axis] = g, r
        for name, nv, vec in (("rcons", abi.RNCONS, abi.RF), ("rprim", RFILL, abi.RH)):
            val = b[name][tuple(src)].copy()
            sg = np.ones(nv)
            if bc == REFLECT:
                sg[vec + d] = -1.0
            if conserved:
                gratio = _ratio(detg[tuple(dst[1:])], detg[tuple(src[1:])])
                for v in range(nv):
                    b[name][(v,) + tuple(dst[1:])] = sg[v] * gratio * val[v]
            else:
                for v in range(nv):
                    b[name][(v,) + tuple(dst[1:])] = sg[v] * val[v]


def _rad_inflow_check(b, ib, jb, kb):
    """phoebus_boundaries.cpp:383-411: no radiation flux into the domain
    through the outer X1 face.  Where H^1 = gamma^1j H_j < 0: H^1 = 0, |H|
    capped at 0.99, H_i = gamma_ij H^j; in the reference's operation order."""
    ks, js, is_ = slice(kb[0], kb[1] + 1), slice(jb[0], jb[1] + 1), slice(ib[0], ib[1] + 1)
    t = b.geom.arrays["cent"][:, js, is_][:, None, :, :]

    def flat(a, c):
        hi, lo = max(a, c), min(a, c)
        return hi * (hi + 1) // 2 + lo

    gcov = [[t[abi.G_GCOV + flat(a + 1, c + 1)] for c in range(3)] for a in range(3)]
    gcon = [[t[abi.G_GAMCON + flat(a, c)] for c in range(3)] for a in range(3)]
    P = b["rprim"]
    H = [P[abi.RH + a, ks, js, is_].copy() for a in range(3)]
    Hcon = []
    for a in range(3):
        acc = np.zeros_like(H[0])
        for c in range(3):
            acc = acc + gcon[a][c] * H[c]
        Hcon.append(acc)
    fix = Hcon[0] < 0.0
    Hcon[0] = np.zeros_like(Hcon[0])
    xi = np.zeros_like(H[0])
    for a in range(3):
        for c in range(3):
            xi = xi + gcov[a][c] * Hcon[a] * Hcon[c]
    xi = np.sqrt(xi)
    cap = xi > 0.99
    with np.errstate(invalid="ignore", divide="ignore"):
        Hcon = [np.where(cap, h * (0.99 / xi), h) for h in Hcon]
    for a in range(3):
        acc = np.zeros_like(H[0])
        for c in range(3):
            acc = acc + gcov[a][c] * Hcon[c]
        P[abi.RH + a, ks, js, is_] = np.where(fix, acc, H[a])


def rad_mesh_exchange(rorc, rp, p, mesh, blocks):
    """The radiation fields' exchange on host blocks, in place, after the
    fluid's (mesh_exchange): neighbours, the boundary functions face by face,
    then ConvertBoundaryConditions' radiation steps (rorc: oracle.RadOracle)."""
    _copy_neighbours(mesh, blocks, [("rcons", range(abi.RNCONS)), ("rprim", range(RFILL))])
    segs = list(mesh.segments())
    for b, seg in zip(blocks, segs):
        for d, outer, bc in _physical_faces(mesh, b, seg):
            _rad_apply_face(b, d, outer, bc, mesh.bc_vars)
    conserved = mesh.bc_vars == abi.BC_VARS_CONSERVED
    for b, seg in zip(blocks, segs):
        faces = _physical_faces(mesh, b, seg)
        if b.geom is not None and p.enable_ox1_fmks_inflow_check and any(d == 0 and o for d, o, _ in faces):
            _rad_inflow_check(b, *_slab(b, 0, True))
        if not conserved:
            for d, outer, _ in faces:
                rorc.MomentPrim2Con(rp, p, b, *_slab(b, d, outer))


def rad_fix_fluxes(p, mesh, blocks):
    """FixFluxes' radiation part (fixup.cpp:728-1078) on the blocks'
    radiation fluxes, in place: on each physical face, over the interior of
    the other axes, reflect zeroes the normal flux of E (X2 faces also F_1,
    F_3), polar the X2 fluxes of E, F_1, F_3; gr_outflow none."""
    if not p.enable_flux_fixup:
        return
    for b, seg in zip(blocks, mesh.segments()):
        (i0, i1), (j0, j1), (k0, k1) = b.interior()
        for d, outer, bc in _physical_faces(mesh, b, seg):
            if bc == REFLECT:
                comps = [abi.RE] + ([abi.RF, abi.RF + 2] if d == 1 else [])
            elif bc == POLAR:
                comps = [abi.RE, abi.RF, abi.RF + 2]
            else:
                continue
            f = b.ng + b.nx[d] if outer else b.ng
            rng = [slice(i0, i1 + 1), slice(j0, j1 + 1), slice(k0, k1 + 1)]
            rng[d] = f
            for m in comps:
                b["rflux"][d * abi.RNCONS + m, rng[2], rng[1], rng[0]] = 0.0

def fix_fluxes_block(p, b, bc_lo, bc_hi):
    """fixup::FixFluxes on one host block's flux array, in place; bc_lo /
    bc_hi: PERIODIC where the face is not on a physical boundary."""
    if not p.enable_flux_fixup:
        return
    F = b["flux"]  # (3 * NCONS, k, j, i): flux(d, m) = F[d * NCONS + m]
    nc = abi.NCONS
    (i0, i1), (j0, j1), (k0, k1) = b.interior()
    ndim = b.ndim
    mhd = bool(p.mhd)

    def f(d, m):
        return F[d * nc + m]

    def clamp(a, upper):  # std::max(F, 0) on upper faces, std::min(F, 0) on lower faces
        if upper:
            a[...] = np.where(a < 0.0, 0.0, a)
        else:
            a[...] = np.where(0.0 < a, 0.0, a)

    ks, js, is_ = slice(k0, k1 + 1), slice(j0, j1 + 1), slice(i0, i1 + 1)
    # x1
    for outer, bc in ((False, bc_lo[0]), (True, bc_hi[0])):
        i = i1 + 1 if outer else i0
        if bc == OUTFLOW:
            clamp(f(0, CRHO)[ks, js, i], outer)
        elif bc == REFLECT:
            f(0, CRHO)[ks, js, i] = 0.0
            f(0, CENG)[ks, js, i] = 0.0
    if ndim == 1:
        return
    for outer, bc in ((False, bc_lo[1]), (True, bc_hi[1])):
        j = j1 + 1 if outer else j0
        if bc == OUTFLOW:
            clamp(f(1, CRHO)[ks, j, is_], outer)
        elif bc == POLAR:
            for m in (CRHO, CENG, CMOM, CMOM + 1, CMOM + 2):
                f(1, m)[ks, j, is_] = 0.0
            if mhd:
                for m in (CB, CB + 1, CB + 2):
                    f(1, m)[ks, j, is_] = 0.0
                src, dst = (j - 1, j) if outer else (j, j - 1)
                f(0, CB + 1)[ks, dst, is_] = -f(0, CB + 1)[ks, src, is_]
                if ndim == 3:
                    f(2, CB + 1)[ks, dst, is_] = -f(2, CB + 1)[ks, src, is_]
        elif bc == REFLECT:
            for m in (CRHO, CENG, CMOM, CMOM + 2):
                f(1, m)[ks, j, is_] = 0.0
    if ndim == 2:
        return
    for outer, bc in ((False, bc_lo[2]), (True, bc_hi[2])):
        k = k1 + 1 if outer else k0
        if bc == OUTFLOW:
            clamp(f(2, CRHO)[k, js, is_], outer)
        elif bc == REFLECT:
            f(2, CRHO)[k, js, is_] = 0.0
            f(2, CENG)[k, js, is_] = 0.0


def block_faces(mesh, seg, b):
    """(bc_lo, bc_hi) of one block: the mesh's kind on a physical face,
    PERIODIC where the block has a neighbour."""
    org = _origin(mesh, seg)
    lo = [mesh.bc_lo[d] if org[d] == 0 else PERIODIC for d in range(3)]
    hi = [mesh.bc_hi[d] if org[d] + b.nx[d] == mesh.n[d] else PERIODIC for d in range(3)]
    return lo, hi


def fix_fluxes(p, mesh, blocks):
    for b, seg in zip(blocks, mesh.segments()):
        lo, hi = block_faces(mesh, seg, b)
        fix_fluxes_block(p, b, lo, hi)


def mesh_stage(orc, p, mesh, blocks, bases, outs, beta, dt):
    """PhoebusDriver::RungeKuttaStage over a tiled mesh on host blocks, in
    the reference's task order: per block sources, fluxes, FluxCT, FixFluxes
    (p.enable_flux_fixup), flux divergence and update into outs; FillDerived
    over the mesh (con2prim, c2p fixup, floors); the boundary exchange of all
    blocks; FillDerived per block again.  blocks[n]['cons'] is the stage
    input."""
    for b, seg, base, out in zip(blocks, mesh.segments(), bases, outs):
        orc.CalculateFluidSourceTerms(p, b)
        orc.CalculateFluxes(p, b)
        orc.FluxCT(p, b)
        lo, hi = block_faces(mesh, seg, b)
        fix_fluxes_block(p, b, lo, hi)
        orc.FluxDivergence(p, b)
        orc.Update(p, b, base, out, beta, dt)
    ins = [b.arrays["cons"] for b in blocks]
    for b, out in zip(blocks, outs):
        b.arrays["cons"] = out
    for _ in range(2):
        if _ == 1:
            mesh_exchange(orc, p, mesh, blocks)
        for b in blocks:
            orc.ConservedToPrimitive(p, b)
            orc.ConservedToPrimitiveFixup(p, b)
            orc.ApplyFloors(p, b)
    for b, c in zip(blocks, ins):
        b.arrays["cons"] = c


def mesh_rk2_step(orc, p, mesh, blocks, seconds, dt):
    """One Heun RK2 step (beta = 1, 1/2) of the mesh on host blocks;
    blocks[n]['cons'] holds U^n on entry and U^{n+1} on exit."""
    bases = [b.arrays["cons"] for b in blocks]
    mesh_stage(orc, p, mesh, blocks, bases, seconds, 1.0, dt)
    for b, s in zip(blocks, seconds):
        b.arrays["cons"] = s
    mesh_stage(orc, p, mesh, blocks, bases, bases, 0.5, dt)
    for b, c in zip(blocks, bases):
        b.arrays["cons"] = c
