"""The reference's function and class names over the generic entry points
(rapidfuzz/distance/*.hpp, rapidfuzz/fuzz.hpp)."""
from ._lib import (DISTANCE, SIMILARITY, NORMALIZED_DISTANCE, NORMALIZED_SIMILARITY, LEVENSHTEIN, INDEL, LCSSEQ,
                   OSA, JARO, JARO_WINKLER, RATIO, PARTIAL_RATIO, TOKEN_SORT_RATIO, PARTIAL_TOKEN_SORT_RATIO,
                   QRATIO, TOKEN_SET_RATIO, PARTIAL_TOKEN_SET_RATIO, TOKEN_RATIO, PARTIAL_TOKEN_RATIO, WRATIO, Cached,
                   Multi, score, editops_many)

__all__ = []


def _free(metric, op, name, has_weights=False, has_pw=False):
    def f(s1, s2, *args, score_cutoff=None, score_hint=None, weights=(1, 1, 1), prefix_weight=0.1):
        a = list(args)
        if has_weights and a:
            weights = a.pop(0)
        if has_pw and a:
            prefix_weight = a.pop(0)
        if a:
            score_cutoff = a.pop(0)
        if a:
            score_hint = a.pop(0)
        return score(metric, op, s1, s2, score_cutoff, score_hint, weights, prefix_weight)
    f.__name__ = name
    globals()[name] = f
    __all__.append(name)


for _metric, _prefix, _w, _pw in ((LEVENSHTEIN, "levenshtein", True, False), (INDEL, "indel", False, False),
                                  (LCSSEQ, "lcs_seq", False, False), (OSA, "osa", False, False),
                                  (JARO, "jaro", False, False), (JARO_WINKLER, "jaro_winkler", False, True)):
    for _op, _suffix in ((DISTANCE, "distance"), (SIMILARITY, "similarity"),
                         (NORMALIZED_DISTANCE, "normalized_distance"), (NORMALIZED_SIMILARITY, "normalized_similarity")):
        _free(_metric, _op, "%s_%s" % (_prefix, _suffix), _w, _pw)


def fuzz_ratio(s1, s2, score_cutoff=0.0):
    return score(RATIO, SIMILARITY, s1, s2, score_cutoff)


__all__.append("fuzz_ratio")


def fuzz_partial_ratio(s1, s2, score_cutoff=0.0):
    """fuzz::partial_ratio (fuzz_impl.hpp:194-239)"""
    return score(PARTIAL_RATIO, SIMILARITY, s1, s2, score_cutoff)


__all__.append("fuzz_partial_ratio")


def fuzz_token_sort_ratio(s1, s2, score_cutoff=0.0):
    """fuzz::token_sort_ratio (fuzz_impl.hpp:297-311)"""
    return score(TOKEN_SORT_RATIO, SIMILARITY, s1, s2, score_cutoff)


def fuzz_partial_token_sort_ratio(s1, s2, score_cutoff=0.0):
    """fuzz::partial_token_sort_ratio (fuzz_impl.hpp:334-349)"""
    return score(PARTIAL_TOKEN_SORT_RATIO, SIMILARITY, s1, s2, score_cutoff)


def fuzz_QRatio(s1, s2, score_cutoff=0.0):
    """fuzz::QRatio (fuzz_impl.hpp:891-909)"""
    return score(QRATIO, SIMILARITY, s1, s2, score_cutoff)


__all__ += ["fuzz_token_sort_ratio", "fuzz_partial_token_sort_ratio", "fuzz_QRatio"]


def _fuzz_free(name, metric, doc):
    def f(s1, s2, score_cutoff=0.0):
        return score(metric, SIMILARITY, s1, s2, score_cutoff)
    f.__name__ = name
    f.__doc__ = doc
    globals()[name] = f
    __all__.append(name)


_fuzz_free("fuzz_token_set_ratio", TOKEN_SET_RATIO, "fuzz::token_set_ratio (fuzz_impl.hpp:422-437)")
_fuzz_free("fuzz_partial_token_set_ratio", PARTIAL_TOKEN_SET_RATIO,
           "fuzz::partial_token_set_ratio (fuzz_impl.hpp:479-495)")
_fuzz_free("fuzz_token_ratio", TOKEN_RATIO, "fuzz::token_ratio (fuzz_impl.hpp:517-571)")
_fuzz_free("fuzz_partial_token_ratio", PARTIAL_TOKEN_RATIO, "fuzz::partial_token_ratio (fuzz_impl.hpp:703-737)")
_fuzz_free("fuzz_WRatio", WRATIO, "fuzz::WRatio (fuzz_impl.hpp:788-829)")


class _CachedBase:
    metric = None

    def __init__(self, s1, *args, **kw):
        self._c = Cached(self.metric, s1, *args, **kw)

    def distance(self, s2, score_cutoff=None, score_hint=None):
        return self._c.score(DISTANCE, s2, score_cutoff, score_hint)

    def similarity(self, s2, score_cutoff=None, score_hint=None):
        return self._c.score(SIMILARITY, s2, score_cutoff, score_hint)

    def normalized_distance(self, s2, score_cutoff=None, score_hint=None):
        return self._c.score(NORMALIZED_DISTANCE, s2, score_cutoff, score_hint)

    def normalized_similarity(self, s2, score_cutoff=None, score_hint=None):
        return self._c.score(NORMALIZED_SIMILARITY, s2, score_cutoff, score_hint)


def _cached(name, metric):
    cls = type(name, (_CachedBase,), {"metric": metric})
    globals()[name] = cls
    __all__.append(name)


for _name, _metric in (("CachedLevenshtein", LEVENSHTEIN), ("CachedIndel", INDEL), ("CachedLCSseq", LCSSEQ),
                       ("CachedOSA", OSA), ("CachedJaro", JARO), ("CachedJaroWinkler", JARO_WINKLER)):
    _cached(_name, _metric)


class CachedRatio:
    def __init__(self, s1):
        self._c = Cached(RATIO, s1)

    def similarity(self, s2, score_cutoff=0.0, score_hint=0.0):
        return self._c.score(SIMILARITY, s2, score_cutoff, score_hint)


__all__.append("CachedRatio")


class CachedPartialRatio:
    """fuzz::CachedPartialRatio (fuzz_impl.hpp:241-283)"""

    def __init__(self, s1):
        self._c = Cached(PARTIAL_RATIO, s1)

    def similarity(self, s2, score_cutoff=0.0, score_hint=0.0):
        return self._c.score(SIMILARITY, s2, score_cutoff, score_hint)


__all__.append("CachedPartialRatio")


def _cached_fuzz(name, metric, doc):
    def __init__(self, s1):
        self._c = Cached(metric, s1)

    def similarity(self, s2, score_cutoff=0.0, score_hint=0.0):
        return self._c.score(SIMILARITY, s2, score_cutoff, score_hint)

    globals()[name] = type(name, (), {"__init__": __init__, "similarity": similarity, "__doc__": doc})
    __all__.append(name)


_cached_fuzz("CachedTokenSortRatio", TOKEN_SORT_RATIO, "fuzz::CachedTokenSortRatio (fuzz_impl.hpp:313-328)")
_cached_fuzz("CachedPartialTokenSortRatio", PARTIAL_TOKEN_SORT_RATIO,
             "fuzz::CachedPartialTokenSortRatio (fuzz_impl.hpp:351-366)")
_cached_fuzz("CachedQRatio", QRATIO, "fuzz::CachedQRatio (fuzz_impl.hpp:911-929)")
_cached_fuzz("CachedTokenSetRatio", TOKEN_SET_RATIO, "fuzz::CachedTokenSetRatio (fuzz_impl.hpp:439-455)")
_cached_fuzz("CachedPartialTokenSetRatio", PARTIAL_TOKEN_SET_RATIO,
             "fuzz::CachedPartialTokenSetRatio (fuzz_impl.hpp:497-513)")
_cached_fuzz("CachedTokenRatio", TOKEN_RATIO, "fuzz::CachedTokenRatio (fuzz_impl.hpp:685-699)")
_cached_fuzz("CachedPartialTokenRatio", PARTIAL_TOKEN_RATIO, "fuzz::CachedPartialTokenRatio (fuzz_impl.hpp:770-784)")
_cached_fuzz("CachedWRatio", WRATIO, "fuzz::CachedWRatio (fuzz_impl.hpp:831-886)")


class experimental:
    """experimental::Multi* (max_len = the MaxLen template argument)"""

    class _MultiBase:
        metric = None

        def __init__(self, max_len, count, *args, **kw):
            self._m = Multi(self.metric, max_len, count, *args, **kw)

        def insert(self, s):
            self._m.insert(s)

        def result_count(self):
            return self._m.result_count()

        def distance(self, s2, score_cutoff=None):
            return self._m.score(DISTANCE, s2, score_cutoff)

        def similarity(self, s2, score_cutoff=None):
            return self._m.score(SIMILARITY, s2, score_cutoff)

        def normalized_distance(self, s2, score_cutoff=None):
            return self._m.score(NORMALIZED_DISTANCE, s2, score_cutoff)

        def normalized_similarity(self, s2, score_cutoff=None):
            return self._m.score(NORMALIZED_SIMILARITY, s2, score_cutoff)

    MultiLevenshtein = type("MultiLevenshtein", (_MultiBase,), {"metric": LEVENSHTEIN})
    MultiIndel = type("MultiIndel", (_MultiBase,), {"metric": INDEL})
    MultiLCSseq = type("MultiLCSseq", (_MultiBase,), {"metric": LCSSEQ})
    MultiOSA = type("MultiOSA", (_MultiBase,), {"metric": OSA})
    MultiJaro = type("MultiJaro", (_MultiBase,), {"metric": JARO})
    MultiJaroWinkler = type("MultiJaroWinkler", (_MultiBase,), {"metric": JARO_WINKLER})

    class MultiRatio(_MultiBase):
        metric = RATIO

        def similarity(self, s2, score_cutoff=0.0):
            return self._m.score(SIMILARITY, s2, score_cutoff)

    class MultiTokenSortRatio(MultiRatio):
        """fuzz::experimental::MultiTokenSortRatio (fuzz.hpp:236-278)"""
        metric = TOKEN_SORT_RATIO

    class MultiQRatio(MultiRatio):
        """fuzz::experimental::MultiQRatio (fuzz.hpp:719-774)"""
        metric = QRATIO


__all__.append("experimental")



def _slice_indices(n, start, stop, step):
    """the positions a slice takes (details/types.hpp:109-135): step must be positive;
    negative bounds count from the end and clamp at 0, bounds past the end clamp to n"""
    if step == 0:
        raise ValueError("slice step cannot be zero")
    if step < 0:
        raise ValueError("step sizes below 0 lead to an invalid order of editops")
    start = max(start + n, 0) if start < 0 else min(start, n)
    stop = max(stop + n, 0) if stop < 0 else min(stop, n)
    return range(start, stop, step) if start < stop else range(0)


_SWAP = {"insert": "delete", "delete": "insert"}


class EditOp(tuple):
    """rapidfuzz::EditOp (details/types.hpp:45-56): (type, src_pos, dest_pos), type one of
    'none', 'replace', 'insert', 'delete'"""
    __slots__ = ()
    _names = ("none", "replace", "insert", "delete")

    def __new__(cls, t, src, dest):
        return tuple.__new__(cls, (cls._names[t], int(src), int(dest)))

    type = property(lambda self: self[0])
    src_pos = property(lambda self: self[1])
    dest_pos = property(lambda self: self[2])


class Editops(list):
    """rapidfuzz::Editops (details/types.hpp:167-...): the operations plus the lengths of
    the source and destination strings"""

    def __init__(self, ops, src_len, dest_len):
        super().__init__(ops)
        self.src_len = src_len
        self.dest_len = dest_len

    def get_src_len(self):
        return self.src_len

    def get_dest_len(self):
        return self.dest_len

    def as_opcodes(self):
        return Opcodes.from_editops(self)

    def slice(self, start, stop, step=1):
        """Editops::slice (details/types.hpp:240-245): the lengths are kept"""
        return Editops([self[i] for i in _slice_indices(len(self), start, stop, step)], self.src_len, self.dest_len)

    def remove_slice(self, start, stop, step=1):
        """Editops::remove_slice (details/types.hpp:247-250, 137-161), in place"""
        drop = set(_slice_indices(len(self), start, stop, step))
        self[:] = [op for i, op in enumerate(self) if i not in drop]

    def reverse(self):
        """Editops::reverse: the operations in reverse order (a new list)"""
        return Editops(self[::-1], self.src_len, self.dest_len)

    def inverse(self):
        """Editops::inverse (details/types.hpp:276-288): the operations turning the
        destination into the source"""
        return Editops([tuple.__new__(EditOp, (_SWAP.get(t, t), d, s)) for t, s, d in self], self.dest_len,
                       self.src_len)

    def remove_subsequence(self, subsequence):
        """Editops::remove_subsequence (details/types.hpp:290-320): the operations left
        once those of subsequence (in order) are taken out, source positions shifted by the
        removed insertions and deletions"""
        if len(subsequence) > len(self):
            raise ValueError("subsequence is not a subsequence")
        out, offset, it = [], 0, 0
        for sop in subsequence:
            while it < len(self) and tuple(self[it]) != tuple(sop):
                t, sp, dp = self[it]
                out.append(tuple.__new__(EditOp, (t, sp + offset, dp)))
                it += 1
            if it == len(self):
                raise ValueError("subsequence is not a subsequence")
            offset += 1 if sop[0] == "insert" else -1 if sop[0] == "delete" else 0
            it += 1
        for t, sp, dp in self[it:]:
            out.append(tuple.__new__(EditOp, (t, sp + offset, dp)))
        return Editops(out, self.src_len, self.dest_len)

    def apply(self, s1, s2):
        """editops_apply (rapidfuzz/distance.hpp:19-60): s1 turned into s2, as a list"""
        out, sp = [], 0
        for t, src, dest in self:
            while sp < src:
                out.append(s1[sp])
                sp += 1
            if t in ("none", "replace"):
                out.append(s2[dest])
                sp += 1
            elif t == "insert":
                out.append(s2[dest])
            else:
                sp += 1
        out.extend(s1[sp:])
        return out


class Opcode(tuple):
    """rapidfuzz::Opcode (details/types.hpp:81-100): (type, src_begin, src_end, dest_begin, dest_end)"""
    __slots__ = ()

    def __new__(cls, t, sb, se, db, de):
        return tuple.__new__(cls, (t, int(sb), int(se), int(db), int(de)))

    type = property(lambda self: self[0])
    src_begin = property(lambda self: self[1])
    src_end = property(lambda self: self[2])
    dest_begin = property(lambda self: self[3])
    dest_end = property(lambda self: self[4])


class Opcodes(list):
    """rapidfuzz::Opcodes: runs of operations, None runs for the unchanged stretches"""

    def __init__(self, ops, src_len, dest_len):
        super().__init__(ops)
        self.src_len = src_len
        self.dest_len = dest_len

    @classmethod
    def from_editops(cls, e):
        """Opcodes(const Editops&) (details/types.hpp:526-569)"""
        out, sp, dp, i = [], 0, 0, 0
        while i < len(e):
            if sp < e[i].src_pos or dp < e[i].dest_pos:
                out.append(Opcode("none", sp, e[i].src_pos, dp, e[i].dest_pos))
                sp, dp = e[i].src_pos, e[i].dest_pos
            sb, db, t = sp, dp, e[i].type
            while True:
                sp += t in ("replace", "delete")
                dp += t in ("replace", "insert")
                i += 1
                if not (i < len(e) and e[i].type == t and e[i].src_pos == sp and e[i].dest_pos == dp):
                    break
            out.append(Opcode(t, sb, sp, db, dp))
        if sp < e.src_len or dp < e.dest_len:
            out.append(Opcode("none", sp, e.src_len, dp, e.dest_len))
        return cls(out, e.src_len, e.dest_len)

    def slice(self, start, stop, step=1):
        """Opcodes::slice (details/types.hpp:429-435): the lengths are kept"""
        return Opcodes([self[i] for i in _slice_indices(len(self), start, stop, step)], self.src_len, self.dest_len)

    def reverse(self):
        """Opcodes::reverse: the runs in reverse order (a new list)"""
        return Opcodes(self[::-1], self.src_len, self.dest_len)

    def inverse(self):
        """Opcodes::inverse (details/types.hpp:461-474)"""
        return Opcodes([Opcode(_SWAP.get(t, t), db, de, sb, se) for t, sb, se, db, de in self], self.dest_len,
                       self.src_len)

    def as_editops(self):
        """Editops(const Opcodes&) (details/types.hpp:500-524)"""
        ops = []
        for t, sb, se, db, de in self:
            if t == "replace":
                ops += [EditOp(1, sb + j, db + j) for j in range(se - sb)]
            elif t == "insert":
                ops += [EditOp(2, sb, db + j) for j in range(de - db)]
            elif t == "delete":
                ops += [EditOp(3, sb + j, db) for j in range(se - sb)]
        return Editops(ops, self.src_len, self.dest_len)

    def apply(self, s1, s2):
        """opcodes_apply (rapidfuzz/distance.hpp:69-103)"""
        out = []
        for t, sb, se, db, de in self:
            if t == "none":
                out.extend(s1[sb:se])
            elif t != "delete":
                out.extend(s2[db:de])
        return out


def _editops(metric, s1, s2, score_hint=None):
    from ._lib import as_units
    a, b = as_units(s1), as_units(s2)
    e = editops_many(metric, [a], [b], score_hint)[0]
    return Editops([EditOp(int(x["type"]), x["src_pos"], x["dest_pos"]) for x in e], a.size, b.size)


def levenshtein_editops(s1, s2, score_hint=None):
    """levenshtein_editops (Levenshtein.hpp:282-295)"""
    return _editops(LEVENSHTEIN, s1, s2, score_hint)


def indel_editops(s1, s2):
    """indel_editops (Indel.hpp:65-75)"""
    return _editops(INDEL, s1, s2)


def lcs_seq_editops(s1, s2):
    """lcs_seq_editops (LCSseq.hpp:65-75)"""
    return _editops(LCSSEQ, s1, s2)


__all__ += ["EditOp", "Editops", "Opcode", "Opcodes", "levenshtein_editops", "indel_editops", "lcs_seq_editops"]
