"""Algorithmic (compulsory) HBM bytes of the kernels of one SIMPLE outer iteration.

Each array a kernel must touch is counted once per launch at its storage width (fp32
values, int32 indices, float4-packed geometry).  Gathers of neighbour values that a
kernel already streams elsewhere are not counted again.  C cells, K faces (Ki internal,
B boundary), F slots per cell, W off-diagonal width, k Krylov iterations.
"""
from __future__ import annotations


def cg_bytes_per_iteration(C: int, W: int, col_bytes: int = 4) -> int:
    """One CG iteration (two passes) per row:
    p = z + beta p_old ; q = A p ; x += alpha_prev p_old :
                   off 4W + col (col_bytes) W + diag 4 + z 4 + p_old 4 + x 8 (rw) + p 4 (w) + q 4 (w)
    r -= alpha q ; z = M r : r 8 (rw) + q 4 + invd 4 + z 4 (w)
    col_bytes 2 when the columns are read as int16 offsets (wcfd_mesh.ell_dcol).
    """
    return C * ((4 + col_bytes) * W + 28 + 20)


def cg_bytes_setup(C: int, W: int, col_bytes: int = 4) -> int:
    """r = b - A x, invd, z, p: off/col (4 + col_bytes) W, diag 4, x 4, b 4, writes r, invd, z, p 16."""
    return C * ((4 + col_bytes) * W + 28)


def cg_bytes(C: int, W: int, iters: int, col_bytes: int = 4) -> int:
    return cg_bytes_setup(C, W, col_bytes) + iters * cg_bytes_per_iteration(C, W, col_bytes)


def bicgstab_bytes_per_iteration(C: int, W: int) -> int:
    """One BiCGSTAB iteration on the 3-component system, per cell (12 B per vector):
    v = A M p : off/col 8W + diag 12 + p 12 + invd 12 + v 12 + r0 12
    s, x      : r 24 + v 12 + x 24 + p 12 + invd 12
    t = A M s : off/col 8W + diag 12 + s 12 + invd 12 + t 12
    x, r      : x 24 + s 12 + invd 12 + t 12 + r 12 + r0 12
    p         : r 12 + p 24 + v 12
    """
    return C * (16 * W + 60 + 84 + 48 + 84 + 48)


def bicgstab_bytes(C: int, W: int, iters: int) -> int:
    setup = C * (8 * W + 12 + 12 + 12 + 12 * 4)
    return setup + iters * bicgstab_bytes_per_iteration(C, W)


def face_pass_bytes(C: int, K: int, Ki: int, B: int, mdot: bool = True) -> int:
    """Every field: internal faces only write their values (16), boundary faces read and
    write them (32) and their gradients."""
    b = 8 * K + 16 * Ki + 16 * K + 16 * B + 64 * C  # owner/nbr, interp, face values, cell values+grads
    b += B * (4 + 4 + 16 + 32 + 4)                   # brow, bc type, bc value, face grads rw, rpf
    if mdot:
        b += 16 * K + 4 * K
    return b


def face_pass_partial_bytes(C: int, K: int, Ki: int, B: int) -> int:
    """One field (the pressure-only pass, no mass flux): face records read and written
    whole (32), the cells' value records (16) and the field's 3 gradient components (12)."""
    return 8 * K + 16 * Ki + 32 * K + 28 * C + B * (4 + 4 + 16 + 16 + 4)


def gradient_bytes(C: int, K: int, F: int, div: bool = False) -> int:
    b = 16 * F * C + 16 * K + 48 * C
    if div:
        b += 4 * K + 4 * C
    return b


def momentum_assembly_bytes(C: int, K: int, F: int, W: int, B: int) -> int:
    return (16 * F * C + 4 * K + 4 * K + 4 * K + B * (4 + 4 + 16 + 16 + 4) + 4 * W * C + 24 * C + 16 * C + 48 * C
            + 4 * C + 4 * C)


def pressure_assembly_bytes(C: int, K: int, F: int, W: int, B: int) -> int:
    return 16 * F * C + 4 * K + 4 * K + 4 * K + B * (4 + 1 + 8) + 4 * W * C + 8 * C + 4 * C


def simple_step_bytes(C, K, Ki, B, F, W, k_u, k_p, n_corr=1, col_bytes=4) -> dict:
    d = {
        "face_pass": face_pass_bytes(C, K, Ki, B) * 2 * n_corr + face_pass_bytes(C, K, Ki, B, mdot=False) * n_corr,
        "gradient": gradient_bytes(C, K, F) + gradient_bytes(C, K, F, div=True) * n_corr
        + gradient_bytes(C, K, F) * n_corr,
        "momentum_assemble": momentum_assembly_bytes(C, K, F, W, B),
        "pressure_assemble": pressure_assembly_bytes(C, K, F, W, B) * n_corr,
        "bicgstab": bicgstab_bytes(C, W, k_u),
        "cg": cg_bytes(C, W, k_p, col_bytes) * n_corr,
        "small": 32 * C + 12 * K,
    }
    d["total"] = sum(d.values())
    return d
