"""Seeded synthetic genomes, reads and assembly graphs for the five workloads.

No public dataset is used: every input is generated here from a seed, with
the shapes the workloads name (genome size, repeat content, coverage, read
length distribution, error profile, k).  Generation is host-side numpy and
sits outside every timed region.

Reads are sampled at uniform random start positions on a random strand and
carry uniform substitution / insertion / deletion errors.  Read ids are Flye
signed ids ``+1 .. +N``; a read's sequence is the forward strand as sampled.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BASES = np.frombuffer(b"ACGT", dtype=np.uint8)
COMP = np.zeros(256, dtype=np.uint8)
for _a, _b in zip(b"ACGTacgtN", b"TGCAtgcaN"):
    COMP[_a] = _b


_COMP_TABLE = bytes(COMP)


def revcomp(seq: np.ndarray) -> np.ndarray:
    """Reverse complement of ASCII bases (a writable copy)."""
    return np.frombuffer(bytearray(seq[::-1].tobytes()).translate(_COMP_TABLE), dtype=np.uint8)


def random_genome(rng: np.random.Generator, length: int) -> np.ndarray:
    return BASES[rng.integers(0, 4, size=length, dtype=np.uint8)]


def mutate(rng: np.random.Generator, seq: np.ndarray, sub: float, ins: float = 0.0,
           dele: float = 0.0) -> np.ndarray:
    """Apply uniform substitution / insertion / deletion errors."""
    n = len(seq)
    out = seq.copy()
    if sub > 0:
        m = rng.random(n) < sub
        shift = rng.integers(1, 4, size=int(m.sum()), dtype=np.uint8)
        code = np.searchsorted(BASES, out[m])
        out[m] = BASES[(code + shift) % 4]
    if ins <= 0 and dele <= 0:
        return out
    r = rng.random(n)
    keep = r >= dele
    insert = (r >= dele) & (r < dele + ins)
    reps = keep.astype(np.int64) + insert.astype(np.int64)
    res = np.repeat(out, reps)
    # the inserted base follows its anchor: positions of anchors after repeat
    ends = np.cumsum(reps)
    ins_pos = ends[insert] - 1
    res[ins_pos] = BASES[rng.integers(0, 4, size=len(ins_pos), dtype=np.uint8)]
    return res


def mutate_sparse(rng: np.random.Generator, seq: np.ndarray, sub: float, ins: float = 0.0,
                  dele: float = 0.0) -> np.ndarray:
    """The error model of `mutate` (each position substituted with
    probability sub, deleted with probability dele, or followed by an inserted
    base with probability ins), drawn as sparse events: the number of each
    kind is binomial and their positions distinct and uniform.  Only the
    touched positions cost random draws, so long reads generate many times
    faster; the random stream differs from `mutate`'s."""
    n = len(seq)
    out = seq.copy()
    if n == 0:
        return out
    ks = int(rng.binomial(n, sub)) if sub > 0 else 0
    if ks:
        pos = rng.choice(n, size=ks, replace=False)
        shift = rng.integers(1, 4, size=ks, dtype=np.uint8)
        code = np.searchsorted(BASES, out[pos])
        out[pos] = BASES[(code + shift) % 4]
    kd = int(rng.binomial(n, dele)) if dele > 0 else 0
    ki = int(rng.binomial(n - kd, ins / (1.0 - dele))) if ins > 0 else 0
    if kd + ki == 0:
        return out
    ev = rng.choice(n, size=kd + ki, replace=False)
    dpos, ipos = np.sort(ev[:kd]), np.sort(ev[kd:])
    kept = np.delete(out, dpos)
    # an inserted base follows its anchor p, which sits at p - (deletions
    # before p) once the deletions are gone
    at = ipos - np.searchsorted(dpos, ipos) + 1
    return np.insert(kept, at, BASES[rng.integers(0, 4, size=ki, dtype=np.uint8)])


def lognormal_lengths(rng, n, mean, sd, lo, hi):
    sigma2 = np.log(1.0 + (sd * sd) / (mean * mean))
    mu = np.log(mean) - sigma2 / 2.0
    v = rng.lognormal(mu, np.sqrt(sigma2), size=n)
    return np.clip(v, lo, hi).astype(np.int64)


@dataclass
class ReadSet:
    ids: np.ndarray  # int64 signed ids
    offsets: np.ndarray  # int64, n+1
    bases: np.ndarray  # uint8 ASCII, concatenated
    # genome start of each read when it was sampled from a genome (else None)
    origin: np.ndarray | None = None

    @property
    def n(self) -> int:
        return len(self.ids)

    @property
    def total_bases(self) -> int:
        return int(self.offsets[-1])

    def seq(self, i: int) -> bytes:
        return self.bases[self.offsets[i]:self.offsets[i + 1]].tobytes()

    def subset(self, idx) -> "ReadSet":
        idx = np.asarray(idx)
        parts = [self.bases[self.offsets[i]:self.offsets[i + 1]] for i in idx]
        lens = np.array([len(p) for p in parts], dtype=np.int64)
        offs = np.zeros(len(idx) + 1, dtype=np.int64)
        offs[1:] = np.cumsum(lens)
        return ReadSet(self.ids[idx].copy(), offs,
                       np.concatenate(parts) if parts else np.zeros(0, np.uint8),
                       None if self.origin is None else self.origin[idx].copy())

    @classmethod
    def from_strings(cls, ids, seqs) -> "ReadSet":
        arrs = [np.frombuffer(s.encode() if isinstance(s, str) else s, dtype=np.uint8)
                for s in seqs]
        offs = np.zeros(len(arrs) + 1, dtype=np.int64)
        offs[1:] = np.cumsum([len(a) for a in arrs])
        return cls(np.asarray(ids, dtype=np.int64), offs,
                   np.concatenate(arrs) if arrs else np.zeros(0, np.uint8))


def sample_reads(rng, genome: np.ndarray, coverage: float, lengths_fn, sub, ins, dele,
                 max_reads: int | None = None, sparse: bool = False) -> ReadSet:
    glen = len(genome)
    target = coverage * glen
    lens: list[np.ndarray] = []
    total = 0
    while total < target:
        chunk = lengths_fn(4096)
        chunk = np.minimum(chunk, glen)
        lens.append(chunk)
        total += int(chunk.sum())
    L = np.concatenate(lens)
    L = L[np.cumsum(L) <= target + L[0]]
    if max_reads is not None:
        L = L[:max_reads]
    n = len(L)
    starts = rng.integers(0, glen - L + 1)
    strand = rng.random(n) < 0.5
    seqs = []
    err = mutate_sparse if sparse else mutate
    for i in range(n):
        s = genome[starts[i]:starts[i] + L[i]]
        if strand[i]:
            s = revcomp(s)
        seqs.append(err(rng, s, sub, ins, dele))
    offs = np.zeros(n + 1, dtype=np.int64)
    offs[1:] = np.cumsum([len(s) for s in seqs])
    return ReadSet(np.arange(1, n + 1, dtype=np.int64), offs, np.concatenate(seqs),
                   np.asarray(starts, dtype=np.int64))


@dataclass
class Workload:
    name: str
    k: int
    reads: ReadSet
    min_freq: int
    max_freq: int
    params: dict = field(default_factory=dict)
    graph: "Graph | None" = None
    seed: int = 0


@dataclass
class Graph:
    edge_ids: np.ndarray  # int64 (> 0)
    seq_ids: np.ndarray  # int64 (> 0) edge-sequence id of each forward edge
    left: np.ndarray  # int32 node ids (complement node = id ^ 1)
    right: np.ndarray
    seqs: ReadSet  # edge sequences, ids = seq_ids


OVERLAP_PARAMS = dict(min_overlap=1000, max_jump=1500, max_gap=500, gap_jump_threshold=100,
                      max_overhang=1500, check_overhang=1, force_local=0, only_max_ext=1,
                      max_overlaps=0, large_gap_penalty=2.0, small_gap_penalty=0.5,
                      min_kmer_survival_rate=0.01, max_divergence=1.0, sample_rate=1.0)


def plain_overlap(seed: int = 1, genome_len: int = 1_000_000, coverage: float = 20.0,
                  max_reads: int | None = None) -> Workload:
    """1 Mb uniform genome, 20x, lognormal(10 kb, 5 kb) in 1-50 kb, 1/0.5/0.5 % errors, k=15."""
    rng = np.random.default_rng(seed)
    genome = random_genome(rng, genome_len)
    reads = sample_reads(rng, genome, coverage,
                         lambda n: lognormal_lengths(rng, n, 10_000, 5_000, 1_000, 50_000),
                         0.01, 0.005, 0.005, max_reads)
    return Workload("plain-1Mb-20x-k15", 15, reads, min_freq=2,
                    max_freq=int(5 * coverage), params=dict(OVERLAP_PARAMS, kmer_size=15),
                    seed=seed)


def repeat_genome(rng, genome_len: int, repeat_len: int, copies: int, repeat_div: float,
                  at_fraction: float) -> np.ndarray:
    genome = random_genome(rng, genome_len)
    rep = random_genome(rng, repeat_len)
    for _ in range(copies):
        pos = int(rng.integers(0, genome_len - repeat_len))
        genome[pos:pos + repeat_len] = mutate(rng, rep, repeat_div)
    at_total = int(at_fraction * genome_len)
    placed = 0
    while placed < at_total:
        ln = int(rng.integers(200, 2001)) & ~1
        pos = int(rng.integers(0, genome_len - ln))
        genome[pos:pos + ln] = np.resize(np.frombuffer(b"AT", dtype=np.uint8), ln)
        placed += ln
    return genome


def batched_repeats(seed: int = 2, genome_len: int = 5_000_000, coverage: float = 40.0,
                    max_reads: int | None = None) -> Workload:
    """5 Mb genome, 30 x 5 kb repeat at 1 % divergence, 2 % (AT)n; HiFi 40x, k=17."""
    rng = np.random.default_rng(seed)
    genome = repeat_genome(rng, genome_len, 5_000, 30, 0.01, 0.02)
    reads = sample_reads(rng, genome, coverage,
                         lambda n: lognormal_lengths(rng, n, 15_000, 3_000, 1_000, 100_000),
                         0.001, 0.0005, 0.0005, max_reads)
    return Workload("batched-5Mb-repeats-40x-k17", 17, reads, min_freq=2,
                    max_freq=int(5 * coverage), params=dict(OVERLAP_PARAMS, kmer_size=17),
                    seed=seed)


def read_to_graph(seed: int = 3, genome_len: int = 20_000_000, n_edges: int = 400,
                  coverage: float = 30.0, max_reads: int | None = None) -> Workload:
    """20 Mb genome cut into 400 edges (log-uniform 5-500 kb), 10 % duplicated at
    0.5 % divergence; ONT 30x lognormal(20 kb, 12 kb) in 1-150 kb, 8 % error, k=15."""
    rng = np.random.default_rng(seed)
    genome = random_genome(rng, genome_len)
    lo, hi = 5_000, 500_000
    raw = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_edges))
    lens = np.maximum((raw / raw.sum() * genome_len).astype(np.int64), 1000)
    lens[-1] = genome_len - lens[:-1].sum()
    cuts = np.concatenate([[0], np.cumsum(lens)])
    seqs = [genome[cuts[i]:cuts[i + 1]] for i in range(n_edges)]
    left = list(range(0, 2 * n_edges, 2))
    right = list(range(2, 2 * n_edges + 2, 2))
    dup = rng.choice(n_edges, size=max(1, n_edges // 10), replace=False)
    for d in sorted(dup):
        seqs.append(mutate(rng, seqs[d], 0.005))
        left.append(left[d])
        right.append(right[d])
    ne = len(seqs)
    offs = np.zeros(ne + 1, dtype=np.int64)
    offs[1:] = np.cumsum([len(s) for s in seqs])
    edge_seqs = ReadSet(np.arange(1, ne + 1, dtype=np.int64), offs, np.concatenate(seqs))
    graph = Graph(np.arange(1, ne + 1, dtype=np.int64), np.arange(1, ne + 1, dtype=np.int64),
                  np.array(left, dtype=np.int32), np.array(right, dtype=np.int32), edge_seqs)
    reads = sample_reads(rng, genome, coverage,
                         lambda n: lognormal_lengths(rng, n, 20_000, 12_000, 1_000, 150_000),
                         0.03, 0.025, 0.025, max_reads)
    params = dict(OVERLAP_PARAMS, kmer_size=15, min_overlap=100, check_overhang=0,
                  max_overhang=0, only_max_ext=0)
    return Workload("read-to-graph-20Mb-400edges-ont30x-k15", 15, reads, min_freq=1,
                    max_freq=64, params=params, graph=graph, seed=seed)


def scale_ont(seed: int = 6, genome_len: int = 500_000_000, coverage: float = 30.0,
              max_reads: int | None = None, sparse_errors: bool = False) -> Workload:
    """The scale configuration's shapes: a genome with 10 % interspersed repeats
    (families of 1-20 kb, copies at 0.5-5 % divergence); ONT-like reads,
    lognormal(25 kb, 15 kb) in 1-150 kb, 6 % error (2 / 2 / 2 % sub / ins /
    del); k = 17.  genome_len and coverage scale it down for tests.
    sparse_errors draws the read errors with `mutate_sparse` (same rates,
    another random stream), for the full-size configuration.

    Solid k-mers are those seen at least max(2, coverage / 10) times: at 30x
    with 6 % error the 15 Gbp of reads fill much of the 4^17 k-mer space with
    erroneous windows, and about 3e9 of those meet once more by chance, so a
    cutoff of 2 would index them all (as Flye's coverage-derived cutoff
    would not)."""
    rng = np.random.default_rng(seed)
    genome = random_genome(rng, genome_len)
    placed = 0
    while placed < 0.10 * genome_len:
        fam = random_genome(rng, int(rng.integers(1_000, 20_001)))
        for _ in range(int(rng.integers(2, 10))):
            pos = int(rng.integers(0, max(1, genome_len - len(fam))))
            copy = mutate(rng, fam, float(rng.uniform(0.005, 0.05)))[:genome_len - pos]
            genome[pos:pos + len(copy)] = copy
            placed += len(copy)
    reads = sample_reads(rng, genome, coverage,
                         lambda n: lognormal_lengths(rng, n, 25_000, 15_000, 1_000, 150_000),
                         0.02, 0.02, 0.02, max_reads, sparse=sparse_errors)
    return Workload("scale-ont30x-k17", 17, reads, min_freq=max(2, int(round(coverage / 10))),
                    max_freq=int(5 * coverage), params=dict(OVERLAP_PARAMS, kmer_size=17),
                    seed=seed)


R2G_PARAMS = dict(max_jump=1500, max_read_overlap=50, min_overlap=1000, max_separation=500,
                  long_edge=900, big_aln=500, max_chain_divergence=0.25)


def small_overlap_case(seed: int, genome_len: int = 60_000, coverage: float = 8.0,
                       mean_len: int = 6_000, k: int = 15, sub=0.01, ins=0.005,
                       dele=0.005, repeat=False) -> Workload:
    """A small seeded overlap workload for parity tests (seconds on the oracle)."""
    rng = np.random.default_rng(seed)
    if repeat:
        genome = repeat_genome(rng, genome_len, 1_500, 6, 0.01, 0.01)
    else:
        genome = random_genome(rng, genome_len)
    reads = sample_reads(rng, genome, coverage,
                         lambda n: lognormal_lengths(rng, n, mean_len, mean_len // 2,
                                                     1_000, 4 * mean_len),
                         sub, ins, dele)
    return Workload(f"small-{seed}", k, reads, min_freq=2, max_freq=int(5 * coverage),
                    params=dict(OVERLAP_PARAMS, kmer_size=k), seed=seed)


def tandem_case(seed: int, genome_len: int = 80_000, coverage: float = 8.0, arrays: int = 3,
                copy_div: float = 0.04, k: int = 15) -> Workload:
    """A small genome carrying tandem arrays (200-350 bp units, 10-16 copies, each
    copy diverged by `copy_div`): a read through an array holds many k-mers two
    or more times below max_freq, so equal keys reach every sort point."""
    rng = np.random.default_rng(seed)
    genome = random_genome(rng, genome_len)
    for a in range(arrays):
        unit = random_genome(rng, int(rng.integers(200, 351)))
        copies = int(rng.integers(10, 17))
        arr = np.concatenate([mutate(rng, unit, copy_div) for _ in range(copies)])
        pos = int((a + 0.5) * genome_len / arrays - len(arr) / 2)
        genome[pos:pos + len(arr)] = arr[:genome_len - pos]
    reads = sample_reads(rng, genome, coverage,
                         lambda n: lognormal_lengths(rng, n, 6_000, 3_000, 1_000, 24_000),
                         0.002, 0.0005, 0.0005)
    return Workload(f"tandem-{seed}", k, reads, min_freq=2, max_freq=int(5 * coverage),
                    params=dict(OVERLAP_PARAMS, kmer_size=k), seed=seed)


@dataclass
class ServingWorkload:
    k: int
    targets: ReadSet  # the genome in 1 Mb pieces (ids 1..n), the served index
    queries: ReadSet  # query pool, ids from 1,000,001
    min_freq: int
    max_freq: int
    params: dict


def serving_workload(seed: int = 4, genome_len: int = 100_000_000, n_queries: int = 2000,
                     piece: int = 1_000_000, k: int = 15) -> ServingWorkload:
    """100 Mb genome with 5 % interspersed repeats (families of 2-8 kb, copies at
    1-3 % divergence), indexed as 1 Mb pieces; queries log-uniform 1-100 kb, half
    HiFi-like (1 % error) and half ONT-like (8 %), from random positions and
    strands."""
    rng = np.random.default_rng(seed)
    genome = random_genome(rng, genome_len)
    placed = 0
    while placed < 0.05 * genome_len:
        fam = random_genome(rng, int(rng.integers(2_000, 8_001)))
        for _ in range(int(rng.integers(3, 12))):
            pos = int(rng.integers(0, genome_len - len(fam)))
            copy = mutate(rng, fam, float(rng.uniform(0.01, 0.03)))[:genome_len - pos]
            genome[pos:pos + len(copy)] = copy
            placed += len(copy)
    npieces = (genome_len + piece - 1) // piece
    targets = ReadSet.from_strings(np.arange(1, npieces + 1),
                                   [genome[i * piece:(i + 1) * piece].tobytes()
                                    for i in range(npieces)])
    lens = np.exp(rng.uniform(np.log(1_000), np.log(100_000), n_queries)).astype(np.int64)
    seqs = []
    for i in range(n_queries):
        ln = int(min(lens[i], genome_len))
        s = int(rng.integers(0, genome_len - ln + 1))
        q = genome[s:s + ln]
        if rng.random() < 0.5:
            q = revcomp(q)
        if rng.random() < 0.5:
            q = mutate(rng, q, 0.005, 0.0025, 0.0025)
        else:
            q = mutate(rng, q, 0.03, 0.025, 0.025)
        seqs.append(q.tobytes())
    queries = ReadSet.from_strings(np.arange(1_000_001, 1_000_001 + n_queries), seqs)
    return ServingWorkload(k, targets, queries, min_freq=1, max_freq=32,
                           params=dict(OVERLAP_PARAMS, kmer_size=k, check_overhang=0,
                                       only_max_ext=0))
