"""The VBR container (reference: src/vbr.py:5-14).

Arrays, as in the reference:
    val     stored block values, each block column-major h x w
    indx    offsets of the blocks in val (n_blocks + 1)
    bindx   block column of each stored block, block-row-major
    rpntr   row partition bounds (n_block_rows + 1)
    cpntr   column partition bounds (n_block_cols + 1)
    bpntrb  first bindx entry of each block row, -1 for an empty row
    bpntre  one past the last bindx entry of each block row, -1 when empty
Lists and numpy arrays are both accepted.
"""
from __future__ import annotations


class VBR:
    def __init__(self, val, indx, bindx, rpntr, cpntr, bpntrb, bpntre):
        self.val = val
        self.indx = indx
        self.bindx = bindx
        self.rpntr = rpntr
        self.cpntr = cpntr
        self.bpntrb = bpntrb
        self.bpntre = bpntre

    def arrays(self):
        return self.val, self.indx, self.bindx, self.rpntr, self.cpntr, self.bpntrb, self.bpntre
