"""Flat npz encoding of block matrices / MPO matrices for the golden fixtures."""
import numpy as np


def pack_bm(prefix, bm, out):
    keys = sorted(bm)
    out[prefix + "_keys"] = np.array(keys, dtype=np.int64).reshape(len(keys), -1)
    out[prefix + "_shapes"] = np.array([bm[k].shape for k in keys], dtype=np.int64).reshape(len(keys), 2)
    out[prefix + "_data"] = np.concatenate([bm[k].ravel(order="F") for k in keys]) if keys else np.zeros(0)


def unpack_bm(prefix, z):
    keys, shapes, data = z[prefix + "_keys"], z[prefix + "_shapes"], z[prefix + "_data"]
    out, off = {}, 0
    for k, (r, c) in zip(keys, shapes):
        out[tuple(int(x) for x in k)] = data[off:off + r * c].reshape((r, c), order="F").copy()
        off += r * c
    return out


def pack_mpo(prefix, w, out):
    terms, Dl, Dr = w
    out[prefix + "_idx"] = np.array([t[:4] for t in terms], dtype=np.int64).reshape(len(terms), 4)
    out[prefix + "_val"] = np.array([t[4] for t in terms], dtype=np.float64)
    out[prefix + "_D"] = np.array([Dl, Dr], dtype=np.int64)


def unpack_mpo(prefix, z):
    idx, val, D = z[prefix + "_idx"], z[prefix + "_val"], z[prefix + "_D"]
    terms = [tuple(int(x) for x in i) + (float(v),) for i, v in zip(idx, val)]
    return (terms, int(D[0]), int(D[1]))


def load_case(z):
    return dict(L=unpack_bm("L", z), R=unpack_bm("R", z), theta=unpack_bm("theta", z), out=unpack_bm("out", z),
                W1=unpack_mpo("W1", z), W2=unpack_mpo("W2", z), ik0=[int(x) for x in z["ik0"]],
                ik1=[int(x) for x in z["ik1"]])
