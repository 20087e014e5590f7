"""CPU restatement of the reference Re_Mesh tool (tools/Re_Mesh/src/mod_remesh.cu).

TEST INFRASTRUCTURE: the oracle of the product's remesh kernel, used only by the
tests.  Pinned against the outputs of the reference tool itself
(tests/golden/remesh.npz, made by tests/golden/make_golden.py remesh).

The tool changes the resolution of a saved field:
  * radial grid of each resolution as init_fd builds it (mod_remesh.cu:60-68, 73-80);
  * the old grid extended by iw points mirrored across the axis (:70-71);
  * per new point r_h[i], i < Nrd-1, Lagrange weights on the 2 iw nearest points of the
    extended grid (Fornberg's algorithm at derivative order 0, fd_weights_rmsh
    :152-178), folded onto the old grid for an even ("+") and an odd ("-") parity
    table RM[2][Nrd][NR] (:85-115); the wall point maps to the old wall point (:83);
  * per old mode (m, l) kept by the new grid (-Ntd/2 <= m < Ntd/2, l < Nzd) the radial
    line is multiplied by the table of its parity -- u_r, u_theta take the even table
    for odd m, u_z for even m (rmsh_k :8-29); every other new mode is zero;
  * mode (0,0): u_r = 0, Im u_theta = 0, Im u_z = 0 at every radius (modeZZ_k :34-40).
"""
import math

import numpy as np

PI2 = 6.283185307179586


def radial_grid(NR):
    """init_fd's wall-clustered grid (mod_remesh.cu:60-68)."""
    N_p = NR + int(math.sqrt(float(NR)))
    r = [0.0] * NR
    for i in range(N_p - NR, N_p):
        ir = N_p - i - 1
        r[i - N_p + NR] = 0.5 * (1.0 + math.cos(0.5 * PI2 * (float(ir) / float(N_p))))
    for _ in range(10):
        dr = 1.5 * r[0] - 0.5 * r[1]
        r = [x * (1.0 + dr) - dr for x in r]
    return r


def lagrange_weights(x, x0):
    """Fornberg's recursion at order 0 (fd_weights_rmsh, mod_remesh.cu:152-178)."""
    n = len(x)
    c = [0.0] * n
    c[0] = 1.0
    c1 = 1.0
    c4 = x[0] - x0
    for i in range(1, n):
        c2 = 1.0
        c5 = c4
        c4 = x[i] - x0
        for j in range(i):
            c3 = x[i] - x[j]
            c2 = c2 * c3
            if j == i - 1:
                c[i] = -c1 * c5 * c[i - 1] / c2
            c[j] = c4 * c[j] / c3
        c1 = c2
    return c


def remesh_matrix(NR, Nrd, iw=3):
    """RM[2][Nrd][NR]: 0 = even folding, 1 = odd folding (mod_remesh.cu:81-115)."""
    r_o, r_h = radial_grid(NR), radial_grid(Nrd)
    rau = [-r_o[iw - i - 1] if i < iw else r_o[i - iw] for i in range(NR + iw)]
    RM = np.zeros((2, Nrd, NR))
    RM[0, Nrd - 1, NR - 1] = 1.0
    RM[1, Nrd - 1, NR - 1] = 1.0
    jleft = 0
    for i in range(Nrd - 1):
        x0 = r_h[i]
        for j in range(NR + iw):
            if rau[j] >= x0:
                jleft = j
                break
        jleft -= iw
        jright = min(NR + iw - 1, jleft + 2 * iw - 1)
        n = jright - jleft + 1
        c = lagrange_weights(rau[jleft:jleft + n], x0)
        jleft -= iw
        jaux = jleft
        for j in range(n):
            if jaux < 0:  # a mirrored point: column iw-j-1, sign by parity (:99-102)
                jcol = iw - j - 1
                jaux += 1
                RM[0, i, jcol] += c[j]
                RM[1, i, jcol] -= c[j]
            else:
                jcol = jleft + j
                RM[0, i, jcol] += c[j]
                RM[1, i, jcol] += c[j]
    return RM


def remesh(fields, new_shape, iw=3):
    """fields: [u_r, u_theta, u_z] complex arrays (NR, NT, NZ) -> the same at new_shape."""
    NR, NT, NZ = fields[0].shape
    Nrd, Ntd, Nzd = new_shape
    RM = remesh_matrix(NR, Nrd, iw)
    out = [np.zeros(new_shape, np.complex128) for _ in range(3)]
    for it in range(NT):
        m = it if it < NT // 2 else it - NT
        if m >= Ntd // 2 or m < -(Ntd // 2):
            continue
        itd = m if m >= 0 else m + Ntd
        L = min(NZ, Nzd)
        for c, flag in ((0, 1), (1, 1), (2, 0)):
            p = abs((abs(m) % 2) - flag)
            out[c][:, itd, :L] = RM[p] @ fields[c][:, it, :L]
    out[0][:, 0, 0] = 0.0
    out[1][:, 0, 0] = out[1][:, 0, 0].real
    out[2][:, 0, 0] = out[2][:, 0, 0].real
    return out
