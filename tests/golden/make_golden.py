"""Generate tests/golden/*.npz from the reference itself.

Runs the reference's own src/vector_database.c + src/kdtree.c (compiled
unmodified into oracle/_ref by oracle/Makefile) through its C API, on seeded
numpy inputs, and stores the inputs' seeds/checksums and the reference's
outputs.  The reference ships no tests, golden vectors or fixtures of its
own; these fixtures are what pins the oracle and the GPU path to it.

    python tests/golden/make_golden.py      (needs the reference sources)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from golden_inputs import (compare_inputs, kd_inputs, mutation_trace, addvec_pairs,  # noqa: E402
                           sha, uuid_trace)


def main() -> None:
    O.build(ref=True)
    ref = O.RefLib()

    # -- /compare metrics on the config-1 shapes (N=10k, D=128 sampled) ----------
    X, pairs = compare_inputs()
    vals = np.empty((pairs.shape[0], 3), np.float32)
    for i, (a, b) in enumerate(pairs):
        for m in range(3):
            vals[i, m] = ref.metric(m, X[a], X[b])
    # adversarial pairs: add_vectors.sh value distribution (test/add_vectors.sh:13-27),
    # odd dimensions, zeros, large magnitudes
    A, B = addvec_pairs()
    adv = np.empty((len(A), 3), np.float32)
    for i in range(len(A)):
        for m in range(3):
            adv[i, m] = ref.metric(m, A[i], B[i])

    # -- /nearest (kdtree_nearest) on config 1: N=10,000 x 128, kd=3 -----------
    Xk, Qk, kd = kd_inputs()
    st = O.RefStore(ref, kd)
    for i in range(Xk.shape[0]):
        st.insert(Xk[i])
    near = np.array([st.nearest(q) for q in Qk], np.int64)

    # -- mutation replay: insert/update/delete, then /nearest + rows ------------
    ops, D2 = mutation_trace()
    st2 = O.RefStore(ref, kd)
    for op, idx, v in ops:
        if op == 0:
            st2.insert(v)
        elif op == 1:
            st2.update(idx, v)
        else:
            st2.delete(idx)
    near_mut = np.array([st2.nearest(q) for q in Qk[:200, :D2]], np.int64)
    size_mut = st2.size
    rows_sha = sha(np.stack([st2.read(i) for i in range(size_mut)]))

    # -- GET /vector?uuid= (vector_db_read_by_uuid) after a uuid trace ----------
    uops, _, ukeys = uuid_trace()
    st3 = O.RefStore(ref, 3)
    for op, idx, v, u in uops:
        if op == 0:
            st3.insert(v, u)
        elif op == 1:
            st3.update(idx, v, u)
        else:
            st3.delete(idx)
    uuid_found = np.array([st3.find_uuid(k) for k in ukeys], np.int64)
    uuid_size = st3.size

    np.savez_compressed(
        os.path.join(HERE, "golden_reference.npz"),
        compare_x_sha=sha(X), compare_pairs_sha=sha(pairs), compare_vals=vals,
        adv_sha=sha(np.concatenate([np.concatenate(A), np.concatenate(B)])), adv_vals=adv,
        kd_x_sha=sha(Xk), kd_q_sha=sha(Qk), kd_nearest=near,
        mut_nearest=near_mut, mut_size=np.int64(size_mut), mut_rows_sha=np.frombuffer(rows_sha.encode(), np.uint8),
        uuid_found=uuid_found, uuid_size=np.int64(uuid_size),
    )
    print("wrote golden_reference.npz:", vals.shape, adv.shape, near.shape, near_mut.shape, size_mut)


if __name__ == "__main__":
    main()
