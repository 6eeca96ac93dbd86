"""slabTree -- drop-in for SslabLU matAssembly/HBS/slabTree.py (tree part).

The spatial bisection tree of the interface points that fixes the HBS leaf
ordering: ``perm_leaf`` (the points of the leaves, leaf by leaf in box-index
order), ``nleaves`` and ``nlevels`` -- the tree protocol the HBS compression
reads (slabTree.py:102-213, 745-751).

Splits (same rules as upstream):
  * line input (points on one line, slabTree.py:25-35): midpoint bisection of
    the interval; a point within 1e-10 of the midpoint belongs to both halves
    (slabTree.py:214-237);
  * rectangle, binary: alternate the split axis by depth -- odd depths split
    x, even depths y -- with the same two-sided tolerance
    (slabTree.py:241-342);
  * rectangle, quad: halve x and y; a point on a split line goes to the lower
    / left child (slabTree.py:549-646).
Children of box b are 2b+1, 2b+2 (binary) or 4b+1..4b+4 (quad: SW, SE, NW,
NE).  A box stops splitting at ``min_leaf_size`` points or at ``max_level``
(rectangles; the line split ignores max_level as upstream does).  Leaves
keep their boundary DOFs (``bDOFs``) and internal boxes their interface DOFs
(``iDOFs``), as upstream leaves them after construction.

Adjacency (slabTree.py:343-547), the near-field structure of the
strong-admissibility HBS: per level, the pairs of boxes that touch --
binary trees by the split-direction rule ('partial', the default) or by a
geometric contact test of the children of touching parents ('full'); quad
trees by the sibling and parent-pair rule -- gathered into
``level_adj_list[l][r]``, the set of level-local ranks adjacent to the box
of rank r at depth l (ranks follow the sorted box indices).

Not built here: the nested interface solve (665-714).
"""
import numpy as np

_TOL = 1e-10


def _is_line(XX, tol=1e-8):
    """slabTree.py:25-35: True when the cloud is (numerically) one line."""
    if XX.shape[1] == 1:
        return True
    Xc = XX - XX.mean(axis=0)
    sv = np.linalg.svd(Xc, compute_uv=False)
    if sv[0] < tol:
        return True
    return float(sv[1] / sv[0]) < tol


class _Node:
    __slots__ = ("index", "level", "bounds", "point_inds", "children", "bDOFs", "iDOFs", "u")

    def __init__(self, index, level, bounds, point_inds):
        self.index = index
        self.level = level
        self.bounds = bounds
        self.point_inds = point_inds
        self.children = []
        self.bDOFs = None
        self.iDOFs = None
        self.u = None

    @property
    def is_leaf(self):
        return len(self.children) == 0


class slabTree:
    """Binary or quad spatial tree over a line or an axis-aligned rectangle."""

    def __init__(self, XX, quad=False, min_leaf_size=1, max_level=np.inf, line_tol=1e-8,
                 adjacency="partial"):
        XX = np.asarray(XX, dtype=float)
        if XX.ndim == 1:
            XX = XX[:, None]
        if XX.ndim != 2:
            raise ValueError("XX must be 1-D or 2-D.")
        self._line = _is_line(XX, tol=line_tol)
        if quad and self._line:
            raise ValueError("quad=True is not valid for line input. Use quad=False, or "
                             "provide a 2-D (rectangle) point cloud.")
        if adjacency not in ("partial", "full"):
            raise ValueError("adjacency must be 'partial' or 'full'.")
        self._XX = XX
        self._quad = quad
        self._adjacency = adjacency
        self._min_leaf_size = min_leaf_size
        self._max_level = max_level
        self._boxes = {}
        # split axes: the coordinates that vary (a plane embedded in 3-D keeps two)
        axes = [d for d in range(XX.shape[1]) if XX[:, d].var() > line_tol]
        self._col_x = int(axes[0])
        self._col_y = int(axes[1]) if len(axes) > 1 else None
        if self._line:
            v = XX[:, self._col_x]
            bounds = (float(v.min()), float(v.max()))
        else:
            x, y = XX[:, self._col_x], XX[:, self._col_y]
            bounds = (float(x.min()), float(x.max()), float(y.min()), float(y.max()))
        root = _Node(0, 0, bounds, np.arange(len(XX)))
        self._boxes[0] = root
        if self._line:
            self._split_line(root)
        elif quad:
            self._split_quad(root)
        else:
            self._split_rect(root)
        self._build_level_adjacency()
        self._build_perm()
        for node in self._boxes.values():
            if not node.is_leaf:
                node.point_inds = None
                node.bDOFs = None

    # ------------------------------------------------------------ construction
    def _add(self, index, level, bounds, inds):
        node = _Node(index, level, bounds, inds)
        self._boxes[index] = node
        return node

    def _split_line(self, root):
        stack = [root]
        while stack:
            box = stack.pop()
            if len(box.point_inds) <= self._min_leaf_size:
                continue
            lo, hi = box.bounds
            mid = 0.5 * (lo + hi)
            v = self._XX[box.point_inds, self._col_x]
            left = self._add(2 * box.index + 1, box.level + 1, (lo, mid),
                             box.point_inds[v <= mid + _TOL])
            right = self._add(2 * box.index + 2, box.level + 1, (mid, hi),
                              box.point_inds[v >= mid - _TOL])
            box.children = [left, right]
            stack += [right, left]

    def _sides(self, pts, bounds, cand):
        """Corner-excluded boundary points of a box among `cand` (indices)."""
        x_lo, x_hi, y_lo, y_hi = bounds
        X = self._XX[cand]
        x, y = X[:, self._col_x], X[:, self._col_y]
        iny = (y > y_lo + _TOL) & (y < y_hi - _TOL)
        inx = (x > x_lo + _TOL) & (x < x_hi - _TOL)
        return {"left": cand[(np.abs(x - x_lo) < _TOL) & iny],
                "down": cand[(np.abs(y - y_lo) < _TOL) & inx],
                "up": cand[(np.abs(y - y_hi) < _TOL) & inx],
                "right": cand[(np.abs(x - x_hi) < _TOL) & iny]}

    def _split_rect(self, box):
        x_lo, x_hi, y_lo, y_hi = box.bounds
        pts = box.point_inds
        if box.level == self._max_level or len(pts) <= self._min_leaf_size:
            box.bDOFs = self._sides(pts, box.bounds, pts)
            return
        split_x = box.level % 2 == 1
        if split_x:
            mid = 0.5 * (x_lo + x_hi)
            v = self._XX[pts, self._col_x]
            lb, rb = (x_lo, mid, y_lo, y_hi), (mid, x_hi, y_lo, y_hi)
        else:
            mid = 0.5 * (y_lo + y_hi)
            v = self._XX[pts, self._col_y]
            lb, rb = (x_lo, x_hi, y_lo, mid), (x_lo, x_hi, mid, y_hi)
        left = self._add(2 * box.index + 1, box.level + 1, lb, pts[v <= mid + _TOL])
        right = self._add(2 * box.index + 2, box.level + 1, rb, pts[v >= mid - _TOL])
        box.children = [left, right]
        self._split_rect(left)
        self._split_rect(right)
        L, R = left.bDOFs, right.bDOFs
        if split_x:
            box.iDOFs = L["right"]
            box.bDOFs = {"left": L["left"], "right": R["right"],
                         "down": np.concatenate([L["down"], R["down"]]),
                         "up": np.concatenate([L["up"], R["up"]])}
        else:
            box.iDOFs = L["up"]
            box.bDOFs = {"left": np.concatenate([L["left"], R["left"]]),
                         "right": np.concatenate([L["right"], R["right"]]),
                         "down": L["down"], "up": R["up"]}

    def _split_quad(self, box):
        x_lo, x_hi, y_lo, y_hi = box.bounds
        pts = box.point_inds
        XX = self._XX
        cx, cy = self._col_x, self._col_y
        if box.level == self._max_level or len(pts) <= self._min_leaf_size:
            # quad leaves search every point for their sides, sorted along them
            sd = self._sides(pts, box.bounds, np.arange(len(XX)))
            box.bDOFs = {"left": sd["left"][np.argsort(XX[sd["left"], cy])],
                         "right": sd["right"][np.argsort(XX[sd["right"], cy])],
                         "down": sd["down"][np.argsort(XX[sd["down"], cx])],
                         "up": sd["up"][np.argsort(XX[sd["up"], cx])]}
            return
        xm, ym = 0.5 * (x_lo + x_hi), 0.5 * (y_lo + y_hi)
        px, py = XX[pts, cx], XX[pts, cy]
        masks = [(px <= xm) & (py <= ym), (px > xm) & (py <= ym),
                 (px <= xm) & (py > ym), (px > xm) & (py > ym)]
        bnds = [(x_lo, xm, y_lo, ym), (xm, x_hi, y_lo, ym), (x_lo, xm, ym, y_hi),
                (xm, x_hi, ym, y_hi)]
        box.children = [self._add(4 * box.index + 1 + q, box.level + 1, b, pts[mk])
                        for q, (mk, b) in enumerate(zip(masks, bnds))]
        for ch in box.children:
            self._split_quad(ch)
        sw, se, nw, ne = box.children
        h = pts[(np.abs(XX[pts, cy] - ym) < _TOL) & (XX[pts, cx] > x_lo + _TOL) &
                (XX[pts, cx] < x_hi - _TOL)]
        h = h[np.argsort(XX[h, cx])]
        v = pts[(np.abs(XX[pts, cx] - xm) < _TOL) & (XX[pts, cy] > y_lo + _TOL) &
                (XX[pts, cy] < y_hi - _TOL)]
        v = v[np.argsort(XX[v, cy])]
        box.iDOFs = np.concatenate([h, v])
        box.bDOFs = {"left": np.concatenate([sw.bDOFs["left"], nw.bDOFs["left"]]),
                     "right": np.concatenate([se.bDOFs["right"], ne.bDOFs["right"]]),
                     "down": np.concatenate([sw.bDOFs["down"], se.bDOFs["down"]]),
                     "up": np.concatenate([nw.bDOFs["up"], ne.bDOFs["up"]])}

    # ------------------------------------------------------------ adjacency
    def _pairs_partial(self):
        """slabTree.py:349-374: siblings touch across the split of their
        parent; of two touching parents, the children facing each other
        touch (one pair when the parents met across this level's split
        direction, two side-by-side pairs otherwise)."""
        out = [[]]
        for lvl in range(1, self.nlevels):
            along = "vertical" if lvl % 2 == 1 else "horizontal"
            across = "horizontal" if along == "vertical" else "vertical"
            cur = [(nd.children[0].index, nd.children[1].index, along)
                   for nd in self.get_nodes_level(lvl - 1)]
            for a, b, d in out[-1]:
                ca, cb = self._boxes[a].children, self._boxes[b].children
                if d == along:
                    cur.append((ca[1].index, cb[0].index, along))
                else:
                    cur.append((ca[0].index, cb[0].index, across))
                    cur.append((ca[1].index, cb[1].index, across))
            out.append(cur)
        return out

    def _touch(self, P, Q, alpha=1e-3):
        """slabTree.py:380-402: boxes touch when the gap along every axis is
        at most alpha times the smaller width there."""
        bp, bq = P.bounds, Q.bounds
        for ax in range(len(bp) // 2):
            lo_p, hi_p, lo_q, hi_q = bp[2 * ax], bp[2 * ax + 1], bq[2 * ax], bq[2 * ax + 1]
            gap = max(lo_p - hi_q, lo_q - hi_p)
            if gap > alpha * min(hi_p - lo_p, hi_q - lo_q):
                return False
        return True

    def _pairs_full(self):
        """slabTree.py:404-441: candidates are siblings and the children of
        touching parents; a candidate is kept when the boxes touch."""
        out = [[]]
        for lvl in range(1, self.nlevels):
            cand = [(nd.children[0], nd.children[1]) for nd in self.get_nodes_level(lvl - 1)
                    if not nd.is_leaf]
            for a, b, _ in out[-1]:
                A, B = self._boxes[a], self._boxes[b]
                if not (A.is_leaf or B.is_leaf):
                    cand += [(p, q) for p in A.children for q in B.children]
            out.append([(p.index, q.index, None) for p, q in cand if self._touch(p, q)])
        return out

    def _pairs_quad(self):
        """slabTree.py:443-489: the four sibling pairs of every split box,
        and the facing children of touching parents."""
        out = [[]]
        for lvl in range(1, self.nlevels):
            cur = []
            for nd in self.get_nodes_level(lvl - 1):
                if nd.is_leaf:
                    continue
                sw, se, nw, ne = (c.index for c in nd.children)
                cur += [(sw, se, "horizontal"), (nw, ne, "horizontal"),
                        (sw, nw, "vertical"), (se, ne, "vertical")]
            for a, b, d in out[-1]:
                A, B = self._boxes[a], self._boxes[b]
                if A.is_leaf or B.is_leaf:
                    continue
                a_sw, a_se, a_nw, a_ne = (c.index for c in A.children)
                b_sw, b_se, b_nw, b_ne = (c.index for c in B.children)
                if d == "horizontal":     # A left of B
                    cur += [(a_se, b_sw, d), (a_ne, b_nw, d)]
                else:                     # A below B
                    cur += [(a_nw, b_sw, d), (a_ne, b_se, d)]
            out.append(cur)
        return out

    def _build_level_adjacency(self):
        """slabTree.py:495-545: level_adj_list from the touching pairs."""
        if self._quad:
            pairs = self._pairs_quad()
        elif self._adjacency == "full":
            pairs = self._pairs_full()
        else:
            pairs = self._pairs_partial()
        self.level_adj_list = []
        for lvl, plist in enumerate(pairs):
            rank = {g: r for r, g in enumerate(self.get_boxes_level(lvl))}
            adj = [set() for _ in rank]
            for a, b, _ in plist:
                adj[rank[a]].add(rank[b])
                adj[rank[b]].add(rank[a])
            self.level_adj_list.append(adj)

    def _build_perm(self):
        """slabTree.py:206-213: leaf point lists, leaves in box-index order."""
        leaves = self.get_leaves()
        parts = [self._boxes[b].point_inds for b in leaves]
        self.perm_leaf = (np.concatenate(parts) if parts else np.zeros(0)).astype(int)

    # ------------------------------------------------------------ queries
    def get_leaves(self):
        return sorted(b.index for b in self._boxes.values() if b.is_leaf)

    def get_boxes_level(self, lvl):
        return sorted(b.index for b in self._boxes.values() if b.level == lvl)

    def get_nodes_level(self, lvl):
        return [b for b in self._boxes.values() if b.level == lvl]

    def get_node(self, idx):
        return self._boxes[idx]

    def get_box_inds(self, box):
        if box not in self._boxes:
            raise KeyError(f"Box {box} does not exist in this tree.")
        return self._boxes[box].point_inds.copy()

    def set_u(self, node, u):
        node.u = u

    @property
    def is_quad(self):
        return self._quad

    @property
    def is_line_input(self):
        return self._line

    @property
    def nlevels(self):
        return max(b.level for b in self._boxes.values()) + 1

    @property
    def nleaves(self):
        return len(self.get_leaves())

    def __repr__(self):
        return ("slabTree(mode=%s, geometry=%s, N=%d, min_leaf_size=%s, depth=%d, n_leaves=%d)"
                % ("quad" if self._quad else "binary", "line" if self._line else "rectangle",
                   len(self._XX), self._min_leaf_size, self.nlevels - 1, self.nleaves))
