"""Oracle-side counterpart of newton.DeviceAssembly for the tests: residual and
FD Jacobian from the CPU oracle, outlet edges added after the bulk in edge
order, Dirichlet rows overwritten -- the same sequence as the device path."""
import numpy as np

from oracle import oracle as O


class OracleAssembly:
    def __init__(self, phys, mesh, rowptr, colind, rows, values, edges=True, nthreads=0):
        self.p, self.m = phys, mesh
        self.rp, self.ci = rowptr, colind
        self.rows, self.values, self.edges = rows, values, edges
        self.nthreads = nthreads

    def set_values(self, values):
        self.values = values

    def __call__(self, TL, EU, want_jac):
        m = self.m
        b, v = O.assemble(self.p, m.conn, m.xyz, TL, EU, self.rp, self.ci, jacobian=want_jac,
                          nthreads=self.nthreads)
        en = m.element_nodes()
        if self.edges:
            for e, ied in m.outlet_edges:
                r, jac, ac = O.edge_open(self.p, m.conn, m.xyz, TL, EU, e, ied, jacobian=want_jac)
                g = en[e]
                for jn in range(9):
                    for je in range(6):
                        row = g[jn] * 6 + je
                        b[row] = b[row] + r[jn, je]
                        if want_jac:
                            cols = self.ci[self.rp[row]:self.rp[row + 1]]
                            for inod in range(9):
                                for ie in range(6):
                                    s = self.rp[row] + np.searchsorted(cols, g[inod] * 6 + ie)
                                    v[s] = v[s] + jac[inod, ie, jn, je]
                            if self.p.nex:
                                s = self.rp[row + 1] - 1
                                v[s] = v[s] + ac[jn, je, 0]
        for r, val in zip(self.rows, self.values):
            b[r] = TL[r % 6, r // 6] - val
            if want_jac:
                s0, s1 = self.rp[r], self.rp[r + 1]
                v[s0:s1] = (self.ci[s0:s1] == r).astype(np.float64)
        return b, (v if want_jac else None)
