"""numpy restatement of the halo planes of a decomposed grid, for the tests: which two
planes a side sends (the interior planes next to it) and receives (its ghost planes),
in the buffer order of the library's pack kernel, ((c nk + k) n_other + o) 2 + t."""
import numpy as np


def planes(n_axis, side, pack):
    """Array offsets (0-based, ghosts included) of the two planes along an axis of
    n_axis entries."""
    if pack:
        return [2, 3] if side == 0 else [n_axis - 4, n_axis - 3]
    return [0, 1] if side == 0 else [n_axis - 2, n_axis - 1]


def as_cpk(field, shape, soa):
    """A 3-component field as a (c, k, j, i) view; shape = (nk, nj, ni)."""
    if soa:
        return field.reshape(3, *shape)
    return np.moveaxis(field.reshape(*shape, 3), 3, 0)


def pack(f4, axis, side):
    """f4: (c, k, j, i) array -> the side's buffer."""
    if axis == 0:
        p = planes(f4.shape[3], side, True)
        return np.ascontiguousarray(f4[:, :, :, p]).ravel()
    p = planes(f4.shape[2], side, True)
    return np.ascontiguousarray(np.transpose(f4[:, :, p, :], (0, 1, 3, 2))).ravel()


def unpack(f4, axis, side, buf):
    nc, nk, nj, ni = f4.shape
    if axis == 0:
        f4[:, :, :, planes(ni, side, False)] = buf.reshape(nc, nk, nj, 2)
    else:
        f4[:, :, planes(nj, side, False), :] = np.transpose(buf.reshape(nc, nk, ni, 2), (0, 1, 3, 2))
