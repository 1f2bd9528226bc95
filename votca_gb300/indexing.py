"""Pair-index convention of the BSE product space (xtp/include/votca/xtp/vc2index.h:36-53).

I(v, c) = ctotal * (v - vmin) + (c - cmin): the virtual index c is the fast one.
"""


class vc2index:
    def __init__(self, vmin, cmin, ctotal):
        self.vmin, self.cmin, self.ctotal = int(vmin), int(cmin), int(ctotal)

    def I(self, v, c):
        return self.ctotal * (v - self.vmin) + (c - self.cmin)

    def v(self, index):
        return index // self.ctotal + self.vmin

    def c(self, index):
        return index % self.ctotal + self.cmin
