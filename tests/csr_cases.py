"""Generated solver-level (CSR) contact problems shared by the oracle and GPU tests."""
import numpy as np


def csr_problem(seed=11, nb=30, nfl=4, nfr=20):
    # a general CSR contact problem (random W rows over two bodies' six columns): its 3x3 Delassus
    # blocks are not diagonal, unlike those of sphere contacts
    rng = np.random.default_rng(seed)
    nv = 6 * nb
    cols, vals, ptr = [], [], [0]
    pairs = [tuple(sorted(rng.choice(nb, 2, replace=False))) for _ in range(nfl + nfr)]
    for u, (a, b) in enumerate(pairs):
        for _ in range(1 if u < nfl else 3):
            for body in (a, b):
                for k in range(6):
                    cols.append(6 * body + k)
                    vals.append(rng.normal())
            ptr.append(len(cols))
    nrows = len(ptr) - 1
    m = rng.uniform(0.5, 2.0, nv)
    return dict(row_ptr=np.array(ptr, np.int32), col=np.array(cols, np.int32), val=np.array(vals),
                contact_bias=rng.normal(size=nrows) * 0.1, mu=rng.uniform(0.1, 0.6, nrows),
                restitution=rng.uniform(0, 0.2, nrows), minv=1.0 / m, mdiag=1.0 / (1.0 / m),
                v=rng.normal(size=nv), f_ext=rng.normal(size=nv), f_gyro=rng.normal(size=nv) * 1e-3, dt=1e-3,
                lam0=np.zeros(nrows), nfl=nfl)
