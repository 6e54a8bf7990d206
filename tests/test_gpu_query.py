"""GPU query lookup against the oracle's querier restatement: per-query matched k-mer
counts over a graph built on the GPU, identical in one batch, one query per launch, and
under the continuous-batching server with Poisson arrivals."""
import numpy as np
import pytest

import oracle
from ggcat_gb300 import _native, serve, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    g = synth.random_genome(150_000, rng)
    gs = [g] + [synth.indels(synth.substitute(g, 0.01, rng), 0.001, 10, rng) for _ in range(2)]
    text, off, ln, _ = synth.pack_sequences(gs)
    ctx = _native.GpuContext(0)
    p = _native.make_params(k=31, m=10, bucket_bits=8, second_bits=2, min_multiplicity=1)
    ctx.build_text(text, p)
    ctx.link(31)
    bases, uo, ul, uf = ctx.unitigs()
    graph = np.frombuffer(_native.unitig_lines(bases, uo, ul), np.uint8).copy()
    d_graph = torch.from_numpy(graph).cuda()
    ctx.query_index(d_graph.data_ptr(), d_graph.numel(), 31)
    r = oracle.build_graph(text, off, ln, oracle.params(k=31, m=10, bucket_bits=8, second_bits=2, threads=4))
    lo, hi, _ = r.kmers()
    queries, arrivals = synth.query_stream(gs, 120, rng, min_len=20, max_len=20_000, rate_per_s=3000.0)
    queries[3] = np.frombuffer(b"ACGTN" * 30, np.uint8)  # N-split query
    queries[4] = np.frombuffer(b"ACG", np.uint8)  # shorter than k
    qt, qo, ql = serve._pack(queries)
    exp, qk, _ = oracle.query(lo, hi, qt, qo, ql, 31)
    yield ctx, queries, arrivals, exp, d_graph
    ctx.close()


def test_query_batch_matches_oracle(setup):
    ctx, queries, arrivals, exp, _ = setup
    text, off, ln = serve._pack(queries)
    ctx.query_submit(0, text, off, ln)
    got = ctx.query_wait(0)
    assert (got == exp).all()
    assert exp.sum() > 0


def test_query_alone_equals_mixed(setup):
    ctx, queries, arrivals, exp, _ = setup
    alone = []
    for i, q in enumerate(queries[:40]):
        text, off, ln = serve._pack([q])
        ctx.query_submit(i % _native.QUERY_SLOTS, text, off, ln)
        alone.append(int(ctx.query_wait(i % _native.QUERY_SLOTS)[0]))
    assert alone == [int(x) for x in exp[:40]]


def test_query_server_continuous_batching(setup):
    ctx, queries, arrivals, exp, _ = setup
    text, off, ln = serve._pack(queries)
    res = serve.serve(ctx, 31, text, off, ln, arrivals, slots=4, max_batch_kmers=200_000)
    assert [int(x) for x in res.matched] == [int(x) for x in exp]
    assert res.batches < len(queries)  # requests were batched together
    base = serve.serve(ctx, 31, text, off, ln, arrivals, slots=4, one_per_launch=True)
    assert [int(x) for x in base.matched] == [int(x) for x in exp]
    assert base.batches == len(queries)


def test_query_graph_from_files_writes_the_querier_csv(setup, tmp_path):
    """GGCATInstance.query_graph on FASTA files: the graph's unitigs indexed on the device,
    one query per FASTA record, and the querier's CSV (query_index, matched_kmers,
    query_kmers = len - (k - 1), matched / query_kmers to two places) with the oracle's
    counts."""
    import ggcat_gb300

    ctx, queries, arrivals, exp, d_graph = setup
    graph = d_graph.cpu().numpy().tobytes()
    gpath, qpath = tmp_path / "graph.fa", tmp_path / "queries.fa"
    with open(gpath, "wb") as f:
        for i, line in enumerate(x for x in graph.split(b"\n") if x):
            f.write(b">%d LN:i:%d\n" % (i, len(line)) + line + b"\n")
    with open(qpath, "wb") as f:
        for i, q in enumerate(queries):
            seq = q.tobytes()
            f.write(b">q%d\n" % i + b"\n".join(seq[j:j + 70] for j in range(0, len(seq), 70)) + b"\n")
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    out = inst.query_graph(str(gpath), str(qpath), str(tmp_path / "result"), kmer_length=31)
    assert out == str(tmp_path / "result.csv")
    rows = open(out).read().strip().split("\n")
    assert rows[0] == "query_index,matched_kmers,query_kmers,match_percentage"
    assert len(rows) == 1 + len(queries)
    for i, row in enumerate(rows[1:]):
        qi, matched, qk, pct = row.split(",")
        n = max(0, len(queries[i]) - 30)
        assert (int(qi), int(matched), int(qk)) == (i, int(exp[i]), n)
        assert pct == ("NaN" if n == 0 else f"{int(exp[i]) / n:.2f}")


def test_query_k63_matches_oracle():
    """k = 63 (u128 index keys): a graph built on the GPU from related genomes, queries with
    substitutions and N, matched counts equal the oracle's."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(63)
    g = synth.random_genome(80_000, rng)
    gs = [g, synth.substitute(g, 0.01, rng)]
    text, off, ln, _ = synth.pack_sequences(gs)
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=63, m=12, bucket_bits=6, second_bits=2, min_multiplicity=1)
        ctx.build_text(text, p)
        ctx.link(63)
        bases, uo, ul, uf = ctx.unitigs()
        graph = np.frombuffer(_native.unitig_lines(bases, uo, ul), np.uint8).copy()
        d_graph = torch.from_numpy(graph).cuda()
        ctx.query_index(d_graph.data_ptr(), d_graph.numel(), 63)
        r = oracle.build_graph(text, off, ln, oracle.params(k=63, m=12, bucket_bits=6, second_bits=2, threads=4))
        lo, hi, _ = r.kmers()
        queries, _ = synth.query_stream(gs, 60, rng, min_len=40, max_len=5_000, rate_per_s=1000.0)
        queries[2] = np.frombuffer(b"ACGTN" * 40, np.uint8)
        qt, qo, ql = serve._pack(queries)
        exp, _, _ = oracle.query(lo, hi, qt, qo, ql, 63)
        ctx.query_submit(0, qt, qo, ql)
        got = ctx.query_wait(0)
        assert (got == exp).all() and exp.sum() > 0
    finally:
        ctx.close()
