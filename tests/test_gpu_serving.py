"""Batched and served proving (lf_prove_batch, lf_submit / lf_poll) against single proofs: the same
seed and table must give the same bytes whether proven alone, in a batch of mixed shapes, or in a
queue mixed with other requests; failures stay per job; admission refuses what exceeds the
context's HBM budget."""
import pytest

pytestmark = pytest.mark.gpu


def _cases(oracle, shapes):
    out = []
    for i, lv in enumerate(shapes):
        seed = bytes([0x30 + i]) * 32
        out.append((seed, lv, oracle.write_table(seed, lv)))
    return out


def test_batch_of_mixed_shapes_matches_single_proofs(prover, gpu_lib, oracle):
    cases = _cases(oracle, [19, 21, 20, 22, 19, 20])
    alone = [prover.prove(s, t, lv) for s, lv, t in cases]
    jobs = [prover.make_job(s, t, lv) for s, lv, t in cases]
    # one job with its table already on the device
    seed, lv, t = cases[2]
    dev = prover.alloc(len(t))
    try:
        prover.h2d(dev, t)
        jobs.append(prover.make_job(seed, dev, lv, on_device=True))
        res = prover.prove_batch(jobs)
    finally:
        prover.free(dev)
    assert [r.status for r in res] == [0] * len(jobs)
    for j, r, want in zip(jobs, res, alone + [alone[2]]):
        assert prover.job_proof(j, r) == want
    ok, msg = oracle.verify(cases[3][0], alone[3], 22, cases[3][2])
    assert ok, msg


MIXED_Q = [661473542593, 9721 * 2917 * 4861, (1 << 64) - 59]


def test_batch_of_mixed_moduli_matches_single_proofs(prover, oracle):
    # Jobs of three moduli interleaved run on both lanes at once: each lane reads its own key's
    # prime constants, so the bytes cannot depend on what the other lane is proving.
    cases = _cases(oracle, [20, 19, 20, 19, 21, 19])
    qs = [MIXED_Q[i % 3] for i in range(len(cases))]
    alone = [prover.prove(s, t, lv, q=q) for (s, lv, t), q in zip(cases, qs)]
    jobs = [prover.make_job(s, t, lv, q=q) for (s, lv, t), q in zip(cases, qs)]
    res = prover.prove_batch(jobs)
    assert [r.status for r in res] == [0] * len(jobs)
    for j, r, want in zip(jobs, res, alone):
        assert prover.job_proof(j, r) == want
    ok, msg = oracle.verify(cases[1][0], alone[1], 19, cases[1][2])
    assert ok, msg


def test_served_mixed_moduli_match_alone(prover, oracle):
    cases = _cases(oracle, [21, 19, 20, 19, 20, 21])
    qs = [MIXED_Q[(i + 1) % 3] for i in range(len(cases))]
    alone = [prover.prove(s, t, lv, q=q) for (s, lv, t), q in zip(cases, qs)]
    jobs = [prover.make_job(s, t, lv, q=q) for (s, lv, t), q in zip(cases, qs)]
    tickets = [prover.submit(j) for j in jobs]
    for j, t, want in zip(jobs, tickets, alone):
        rc, r = prover.poll(t, 60000)
        assert rc == 0 and r.status == 0
        assert prover.job_proof(j, r) == want


def test_budget_for_one_request_serialises_the_queue(gpu_lib, oracle):
    # A budget that holds one 2^21 request but not two: the second starts only after the first
    # has finished (its queueing time covers the first's run), and both proofs are unchanged.
    cases = _cases(oracle, [21, 21])
    with gpu_lib.Prover(0) as free:
        alone = [free.prove(s, t, lv) for s, lv, t in cases]
        need = free.footprint(21)
    with gpu_lib.Prover(0, hbm_budget=need + need // 2) as p:
        jobs = [p.make_job(s, t, lv) for s, lv, t in cases]
        tickets = [p.submit(j) for j in jobs]
        res = []
        for j, t, want in zip(jobs, tickets, alone):
            rc, r = p.poll(t, 60000)
            assert rc == 0 and r.status == 0
            assert p.job_proof(j, r) == want
            res.append(r)
        assert res[1].queue_ms >= res[0].run_ms * 0.9


def test_batch_failure_stays_with_its_job(prover, oracle):
    cases = _cases(oracle, [19, 20])
    good = [prover.make_job(s, t, lv) for s, lv, t in cases]
    bad = prover.make_job(b"\x05" * 32, cases[0][2][:-16], 19)  # one word short
    res = prover.prove_batch([good[0], bad, good[1]])
    assert res[1].status == -4  # LF_E_TABLE_LEN
    assert res[0].status == 0 and res[2].status == 0
    assert prover.job_proof(good[1], res[2]) == prover.prove(cases[1][0], cases[1][2], 20)


def test_served_requests_match_alone_and_tickets_retire(prover, gpu_lib, oracle):
    cases = _cases(oracle, [22, 19, 20, 19, 21])
    alone = [prover.prove(s, t, lv) for s, lv, t in cases]
    jobs = [prover.make_job(s, t, lv) for s, lv, t in cases]
    tickets = [prover.submit(j) for j in jobs]
    rc, early = prover.poll(tickets[-1], 0)  # just looking: done (result taken) or still pending
    assert rc in (0, gpu_lib.LF_E_TIMEOUT)
    if rc == 0:
        assert early.status == 0 and prover.job_proof(jobs[-1], early) == alone[-1]
        jobs, tickets, alone = jobs[:-1], tickets[:-1], alone[:-1]
    for j, t, want in zip(jobs, tickets, alone):
        rc, r = prover.poll(t, 60000)
        assert rc == 0 and r.status == 0
        assert prover.job_proof(j, r) == want
        assert r.queue_ms >= 0 and r.run_ms > 0
        assert prover.poll(t, 0)[0] == -12  # retired
    assert prover.poll(10 ** 9, 0)[0] == -12  # never issued


def test_admission_against_the_hbm_budget(gpu_lib, oracle):
    with gpu_lib.Prover(0, hbm_budget=64 << 20) as small:
        seed = b"\x07" * 32
        table = oracle.write_table(seed, 19)
        assert small.prove(seed, table, 19)  # fits
        big = small.make_job(seed, 1 << 12, 31, nbytes=(1 << 31) // 8)  # never dereferenced
        with pytest.raises(gpu_lib.LfError) as e:
            small.submit(big)
        assert e.value.code == -9  # LF_E_ADMISSION


def test_lane_count_is_checked_and_one_lane_batches_match(gpu_lib, oracle):
    with pytest.raises(gpu_lib.LfError) as e:
        gpu_lib.Prover(0, lanes=9)
    assert e.value.code == gpu_lib.LF_E_ARGS
    cases = _cases(oracle, [19, 20, 19])
    with gpu_lib.Prover(0) as many, gpu_lib.Prover(0, lanes=1) as one:
        want = [many.prove(s, t, lv) for s, lv, t in cases]
        for p in (many, one):
            jobs = [p.make_job(s, t, lv) for s, lv, t in cases]
            res = p.prove_batch(jobs)
            assert [p.job_proof(j, r) for j, r in zip(jobs, res)] == want
        assert many.footprint(20) > many.footprint(19) > many.footprint(19, host_table=False) > 0
        assert many.footprint(18) == 0  # unsupported shape
