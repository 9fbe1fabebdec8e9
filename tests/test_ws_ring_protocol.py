"""Model check of the warp-specialised convolution's mbarrier protocol
(conv3x3_umma_ws_kernel in vulkanpbrt_gb300/csrc/nn_umma.cu), on the CPU.

The roles run the kernel's loops with its index formulas (stage i % stages,
phase i / stages, accumulator buffer i & 1, gather-warp ownership
(i % stages) % 4 == warp) against barriers with the hardware's
try_wait.parity rule (a wait on parity p passes while the barrier's current
phase has the other parity). The asynchronous completions (TMA loads, MMA
commits) fire at random later points, TMA loads in any order, MMA commits
in issue order. Every wait that passes is checked against what it is meant
to guarantee: the stage holds this tile's data (all parts), a stage is not
refilled while MMAs still read it, an accumulator buffer is drained before
it is reused and holds this tile's result when drained. Random schedules
cover 2-6 stages, with and without the TMA producer and the gather warps,
the FP8 form (the TMA completing on its own barrier, the gather warp
quantising after it), and the TMA load of the second input's
half-resolution box (completing on its own barrier; the gather warp expands
it into the stage's planes, and the producer must not refill the box while
the gather warp reads it). The superseded ownership rule (gather warp i % 4,
which let two warps share a stage when there were fewer stages than gather
warps) is checked to fail, so the model is shown to catch that fault."""
import random

import pytest

GATHER_WARPS = 4


class Barrier:
    def __init__(self, count):
        self.count = count
        self.pending = count
        self.phase = 0  # completed phases

    def arrive(self):
        self.pending -= 1
        assert self.pending >= 0, "more arrivals than the barrier's count"
        if self.pending == 0:
            self.phase += 1
            self.pending = self.count

    def passes(self, parity):
        return (self.phase & 1) != parity


class Violation(AssertionError):
    pass


def run(stages, tiles, tma, gather, fp8, owner, rng, stg=False, gather_all=False):
    """One random schedule of one CTA's roles over `tiles` tiles. Raises Violation on a broken guarantee,
    returns False on a deadlock (no role can move), True when every role finished."""
    # gather_all: every gather warp fills part of every stage and arrives on it
    # (the backward-weights kernel); else each stage has one owning warp
    n_arrive = GATHER_WARPS if gather_all else 1
    full = [Barrier((0 if fp8 else (1 if tma else 0)) + (n_arrive if gather else 0)) for _ in range(stages)]
    empty = [Barrier(1) for _ in range(stages)]
    tmab = [Barrier(1) for _ in range(stages)]  # FP8: the TMA's own barrier
    stgb = [Barrier(1) for _ in range(stages)]  # the half-resolution box's barrier
    stg_part = [None] * stages
    expanding = [False] * stages
    tfull = [Barrier(1) for _ in range(2)]
    tempty = [Barrier(1) for _ in range(2)]
    # stage contents: which tile's TMA part / gathered part is in place; MMAs reading the stage
    tma_part = [None] * stages
    gat_part = [None] * stages
    converted = [None] * stages
    readers = [0] * stages
    acc = [None, None]  # tile whose result sits in accumulator buffer b
    drained = [-2, -1]  # last tile drained from buffer b
    inflight_tma = []  # (stage, tile)
    inflight_mma = []  # (stage, buffer, tile), completes in order

    def producer():
        for i in range(tiles):
            st, k = i % stages, i // stages
            while not empty[st].passes((k & 1) ^ 1):
                yield
            if readers[st]:
                raise Violation(f"TMA refills stage {st} for tile {i} while MMAs read it")
            if expanding[st]:
                raise Violation(f"TMA refills stage {st}'s box for tile {i} while the gather warp expands it")
            inflight_tma.append((st, i, "x1"))
            if stg:
                inflight_tma.append((st, i, "x2"))
            yield

    gat_parts = [set() for _ in range(stages)]  # gather_all: which warps filled the stage for its tile

    def gatherer(gw):
        for i in range(tiles):
            if not gather_all and owner(i, stages) != gw:
                continue
            st, k = i % stages, i // stages
            while not empty[st].passes((k & 1) ^ 1):
                yield
            if readers[st]:
                raise Violation(f"gather warp {gw} refills stage {st} for tile {i} while MMAs read it")
            if gather_all:
                if gat_part[st] != i:
                    gat_part[st] = i
                    gat_parts[st] = set()
                gat_parts[st].add(gw)
            else:
                gat_part[st] = i
            yield
            if stg:
                while not stgb[st].passes(k & 1):
                    yield
                if stg_part[st] != i:
                    raise Violation(f"tile {i}: expanded stage {st} before its box landed")
                expanding[st] = True
                yield
                expanding[st] = False
            if fp8:
                if tma:
                    while not tmab[st].passes(k & 1):
                        yield
                    if tma_part[st] != i:
                        raise Violation(f"tile {i}: quantised stage {st} before its TMA part landed")
                converted[st] = i
            full[st].arrive()
            yield

    def mma():
        for i in range(tiles):
            st, k, b, kb = i % stages, i // stages, i & 1, i >> 1
            while not full[st].passes(k & 1):
                yield
            if tma and tma_part[st] != i:
                raise Violation(f"MMA of tile {i}: stage {st} holds TMA part of tile {tma_part[st]}")
            if gather and gat_part[st] != i:
                raise Violation(f"MMA of tile {i}: stage {st} holds gathered part of tile {gat_part[st]}")
            if gather_all and len(gat_parts[st]) != GATHER_WARPS:
                raise Violation(f"MMA of tile {i}: stage {st} filled by warps {sorted(gat_parts[st])} only")
            if stg and stg_part[st] != i:
                raise Violation(f"MMA of tile {i}: stage {st} expanded from the box of tile {stg_part[st]}")
            if fp8 and converted[st] != i:
                raise Violation(f"MMA of tile {i}: stage {st} not quantised")
            while not tempty[b].passes((kb & 1) ^ 1):
                yield
            if drained[b] != i - 2:
                raise Violation(f"MMA of tile {i} into buffer {b} before tile {i - 2} was drained")
            readers[st] += 1
            inflight_mma.append((st, b, i))
            yield

    def epilogue():
        for i in range(tiles):
            b, kb = i & 1, i >> 1
            while not tfull[b].passes(kb & 1):
                yield
            if acc[b] != i:
                raise Violation(f"epilogue of tile {i} reads buffer {b} holding tile {acc[b]}")
            acc[b] = None
            drained[b] = i
            yield
            tempty[b].arrive()
            yield

    roles = []
    if tma:
        roles.append(producer())
    if gather:
        roles += [gatherer(gw) for gw in range(GATHER_WARPS)]
    roles += [mma(), epilogue()]
    live = list(roles)

    def complete_tma():
        j = rng.randrange(len(inflight_tma))
        st, i, part = inflight_tma.pop(j)
        if part == "x2":
            stg_part[st] = i
            stgb[st].arrive()
            return
        tma_part[st] = i
        (tmab if fp8 else full)[st].arrive()

    def complete_mma():
        st, b, i = inflight_mma.pop(0)
        readers[st] -= 1
        acc[b] = i
        empty[st].arrive()
        tfull[b].arrive()

    stuck = 0
    while live or inflight_tma or inflight_mma:
        choices = [("role", r) for r in live]
        if inflight_tma:
            choices.append(("tma", None))
        if inflight_mma:
            choices.append(("mma", None))
        kind, r = rng.choice(choices)
        if kind == "tma":
            complete_tma()
            stuck = 0
        elif kind == "mma":
            complete_mma()
            stuck = 0
        else:
            before = (len(inflight_tma), len(inflight_mma),
                      [b.phase for b in full + empty + tmab + stgb + tfull + tempty], list(expanding))
            try:
                next(r)
            except StopIteration:
                live.remove(r)
            after = (len(inflight_tma), len(inflight_mma),
                     [b.phase for b in full + empty + tmab + stgb + tfull + tempty], list(expanding))
            stuck = stuck + 1 if before == after else 0
        if stuck > 20000:
            return False
    return True


def owner_kernel(i, stages):
    return (i % stages) % GATHER_WARPS


def owner_round_robin(i, stages):  # the superseded rule
    return i % GATHER_WARPS


@pytest.mark.parametrize("stages", [2, 3, 4, 5, 6])
@pytest.mark.parametrize("tma,gather,fp8", [(True, False, False), (True, True, False), (False, True, False),
                                            (True, True, True), (False, True, True)])
def test_ring_protocol_holds(stages, tma, gather, fp8):
    rng = random.Random(stages * 7 + tma * 3 + gather * 5 + fp8 * 11)
    for _ in range(150):
        tiles = rng.randrange(1, 4 * stages + 6)
        assert run(stages, tiles, tma, gather, fp8, owner_kernel, rng), "deadlock"


@pytest.mark.parametrize("stages", [2, 3, 4, 5, 6])
@pytest.mark.parametrize("fp8", [False, True])
def test_ring_protocol_holds_with_box(stages, fp8):
    rng = random.Random(stages * 13 + fp8)
    for _ in range(150):
        tiles = rng.randrange(1, 4 * stages + 6)
        assert run(stages, tiles, True, True, fp8, owner_kernel, rng, stg=True), "deadlock"


@pytest.mark.parametrize("stages", [2, 3, 4])
def test_ring_protocol_holds_with_every_warp_on_every_stage(stages):
    """The backward-weights kernel's form: the gather warps all fill part of
    every stage, each arriving on its full barrier (count 1 + warps)."""
    rng = random.Random(stages * 17)
    for _ in range(200):
        tiles = rng.randrange(1, 4 * stages + 6)
        assert run(stages, tiles, True, True, False, owner_kernel, rng, gather_all=True), "deadlock"


def test_model_catches_shared_stage_ownership():
    rng = random.Random(1)
    with pytest.raises(Violation):
        for _ in range(3000):
            run(2, 12, True, True, False, owner_round_robin, rng)
