"""Row-by-row meaning of filter expressions, written from the symbol semantics alone.

A sequence leaf asks for the symbol a row's aligned sequence holds at a position (the missing
symbol N / X where the row is not covered); a row without a sequence matches no symbol. The
ambiguity modes follow the reference's rewrite rules (Maybe -> upper bound, Exact -> lower bound,
Not flips the mode, an exact NOf under a non-default mode becomes at-least-n and not
at-least-n+1). This is independent of storage, containers, coverage indexes and operator trees,
and is used to cross-check the oracle and the planner on small tables.
"""
from __future__ import annotations

import numpy as np

NUC = "-ACGTRYSWKMBDHVN"
AA = "-ACDEFGHIKLMNOPQRSTUVWYBJZ*X"


def _codes(kind):
    if kind == 0:
        c = {s: {s} for s in "-ACGT"}
        c.update({"R": set("AG"), "Y": set("CT"), "S": set("GC"), "W": set("AT"), "K": set("GT"), "M": set("AC"),
                  "B": set("CGT"), "D": set("AGT"), "H": set("ACT"), "V": set("ACG"), "N": set(NUC)})
        return NUC, c
    c = {s: {s} for s in AA}
    c.update({"B": set("DN"), "J": set("LI"), "Z": set("QE"), "X": set(AA)})
    return AA, c


def ambiguity(kind):
    alpha, codes = _codes(kind)
    return {s: {y for y in alpha if codes[s] <= codes[y]} for s in alpha}


class Column:
    def __init__(self, name, kind, reference, rows):
        self.name, self.kind, self.reference = name, kind, reference
        self.alpha = NUC if kind == 0 else AA
        self.missing = "N" if kind == 0 else "X"
        self.null = np.array([r is None for r in rows])
        L = len(reference)
        idx = {c: i for i, c in enumerate(self.alpha)}
        if kind == 0:
            idx.update({"U": idx["T"]})
        self.sym = np.zeros((len(rows), L), np.int8)
        for i, r in enumerate(rows):
            s = reference if r is None else r
            self.sym[i] = [idx[ch.upper()] for ch in s]
        self.amb = ambiguity(kind)


def parse(text):
    i = 0

    def ws():
        nonlocal i
        while i < len(text) and text[i] == " ":
            i += 1

    def tok():
        nonlocal i
        ws()
        j = i
        while i < len(text) and text[i] not in ",()":
            i += 1
        return text[j:i].strip()

    def eat(c):
        nonlocal i
        ws()
        if i < len(text) and text[i] == c:
            i += 1
            return True
        return False

    def node():
        name = tok()
        if name in ("True", "False"):
            return (name,)
        assert eat("(")
        args = []
        if name in ("And", "Or"):
            if not eat(")"):
                args.append(node())
                while eat(","):
                    args.append(node())
                assert eat(")")
            return (name, args)
        if name in ("Not", "Maybe", "Exact"):
            a = node()
            assert eat(")")
            return (name, a)
        if name == "NOf":
            n = int(tok())
            assert eat(",")
            mode = tok()
            kids = []
            while eat(","):
                kids.append(node())
            assert eat(")")
            return (name, n, mode == "exactly", kids)
        while True:
            args.append(tok())
            if eat(")"):
                break
            assert eat(",")
        return (name, *args)

    return node()


UPPER, LOWER, NONE = "upper", "lower", "none"


def _invert(m):
    return {UPPER: LOWER, LOWER: UPPER}.get(m, m)


class Table:
    def __init__(self, n_rows, columns, dicts, dates):
        self.n = n_rows
        self.cols = {c.name: c for c in columns}
        self.dicts = dicts  # name -> list of values / None
        self.dates = dates  # name -> np.int64 array, None -> INT32_MIN

    def evaluate(self, text):
        return self._ev(parse(text), NONE)

    def _ev(self, e, mode):
        k = e[0]
        if k == "True":
            return np.ones(self.n, bool)
        if k == "False":
            return np.zeros(self.n, bool)
        if k == "And":
            r = np.ones(self.n, bool)
            for c in e[1]:
                r &= self._ev(c, mode)
            return r
        if k == "Or":
            r = np.zeros(self.n, bool)
            for c in e[1]:
                r |= self._ev(c, mode)
            return r
        if k == "Not":
            return ~self._ev(e[1], _invert(mode))
        if k == "Maybe":
            return self._ev(e[1], UPPER)
        if k == "Exact":
            return self._ev(e[1], LOWER)
        if k == "NOf":
            _, n, exact, kids = e
            cnt = np.zeros(self.n, np.int64)
            for c in kids:
                cnt += self._ev(c, mode)
            if mode != NONE and exact and n < len(kids):
                return (cnt >= n) & ~(cnt >= n + 1)
            return cnt == n if exact else cnt >= n
        if k in ("SymEq", "HasMut"):
            col = self.cols[e[1]]
            p = int(e[2]) - 1
            ref = col.reference[p].upper()
            if k == "SymEq":
                c = ref if e[3] == "." else e[3].upper()
                if col.kind == 0 and c == "U":
                    c = "T"
                S = col.amb[c] if mode == UPPER else {c}
            else:
                S = set(col.alpha) - ({ref} if mode == UPPER else col.amb[ref])
            ids = [col.alpha.index(s) for s in S]
            return ~col.null & np.isin(col.sym[:, p], ids)
        if k in ("MutProfile", "MutProfileMutations"):
            # at most `distance` positions whose symbol is not compatible with the profile's
            # (not in its ambiguity set; positions where the profile is missing never count);
            # a row without a sequence differs nowhere
            col = self.cols[e[1]]
            dist = int(e[2])
            if k == "MutProfile":
                prof = e[3].upper()
            else:
                prof = list(col.reference.upper())
                for m in e[3:]:
                    pos, sym = m.split(":")
                    prof[int(pos) - 1] = sym.upper()
            cnt = np.zeros(self.n, np.int64)
            for p, c in enumerate(prof):
                if col.kind == 0 and c == "U":
                    c = "T"
                if c == col.missing:
                    continue
                ok = [col.alpha.index(y) for y in col.amb[c]]
                cnt += ~np.isin(col.sym[:, p], ok)
            cnt[col.null] = 0
            return cnt <= dist
        if k == "StrEq":
            vals = self.dicts[e[1]]
            return np.array([v == e[2] for v in vals])
        if k == "DateBetween":
            d = self.dates[e[1]]
            lo = -(2 ** 31) if e[2] == "*" else int(e[2])
            hi = 2 ** 31 - 1 if e[3] == "*" else int(e[3])
            return (d != -(2 ** 31)) & (d >= lo) & (d <= hi)
        raise ValueError(k)


def from_raw(raw) -> Table:
    """Semantic table from a rhydb_gpu.RawTable (aligned sequences reconstructed from the runs)."""
    n = raw.n_rows
    cols = []
    for c in range(raw.n_seq):
        s = raw.seq[c]
        ref = s.reference[: s.L].decode()
        rows = []
        for r in range(n):
            if s.is_null[r]:
                rows.append(None)
                continue
            chars = list(ref)
            for k in range(s.row_off[r], s.row_off[r + 1]):
                ch = s.run_char[k].decode()
                for p in range(s.run_pos[k], s.run_pos[k] + s.run_len[k]):
                    chars[p] = ch
            rows.append("".join(chars))
        cols.append(Column(s.name.decode(), s.kind, ref, rows))
    dicts = {}
    for c in range(raw.n_dict):
        d = raw.dict[c]
        vals = [d.values[i].decode() for i in range(d.n_values)]
        dicts[d.name.decode()] = [None if d.ids[r] == 0xFFFFFFFF else vals[d.ids[r]] for r in range(n)]
    dates = {}
    for c in range(raw.n_date):
        d = raw.date[c]
        dates[d.name.decode()] = np.array([d.days[r] for r in range(n)], np.int64)
    return Table(n, cols, dicts, dates)


def profile_queries(sem, rng):
    """MutationProfile queries: near a row's own sequence, the reference with mutations, missing
    and ambiguous profile symbols, distances 0 .. 50."""
    col = sem.cols["main"]
    L = len(col.reference)
    out = []
    rows = rng.choice(np.flatnonzero(~col.null), 4, replace=False)
    for i, r in enumerate(rows):
        prof = [col.alpha[x] for x in col.sym[r]]
        for p in rng.choice(L, 3 * i, replace=False):
            prof[p] = "ACGTN-RY"[rng.integers(8)]
        for d in (0, 1, 5, 50):
            out.append(f"MutProfile(main,{d},{''.join(prof)})")
    out.append(f"MutProfile(main,0,{'N' * L})")
    out.append(f"MutProfile(main,3,{col.reference.lower()})")
    muts = ",".join(f"{p + 1}:{'ACGTN'[p % 5]}" for p in rng.choice(L, 12, replace=False))
    for d in (0, 2, 12, 200):
        out.append(f"MutProfileMutations(main,{d},{muts})")
    out.append("MutProfileMutations(main,0)")
    out.append("Not(MutProfileMutations(ORF1a,1,5:K,7:X))")
    out.append(f"And(StrEq(country,country_001),MutProfileMutations(main,4,{muts}))")
    return out
