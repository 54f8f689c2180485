"""The classified Proth/Riesel/Mersenne path keeps about 61 bytes of class
buffers per prime of a segment (codes, items, refinement lists, the eight
pattern lists).  Where the device cannot give them, the residue launch walks
every term instead -- the same factors, no error.  Checked here by filling
the device's free memory with a PyTorch tensor, leaving less than those
buffers need, and comparing the run with the term-by-term walk's factor file
(integers: the comparison is exact)."""
import pytest

import cutrialdive_gb300 as ctd
import oracle as O

pytestmark = pytest.mark.gpu

SEG = 1 << 29
# primes below 2^32 + 2^29 in the segment, bounded below (p / ln p with
# ln p < 22.5): each needs about 61 bytes of class buffers
MIN_PRIMES = SEG * 2 // 45


def run(eng, variant):
    t = eng.get_tuning(O.PROTH)
    t["variant"] = variant
    eng.set_tuning(O.PROTH, t)
    job = ctd.CtdJob(O.PROTH, 32, 3, 1, 100001, 1 << 32, (1 << 32) + SEG)
    buf = ctd.factors_buffer.empty(1, 100000, 32)
    eng.run_plain(job, buf, segment_length=SEG)
    return buf


def test_classified_path_without_room_for_its_buffers():
    torch = pytest.importorskip("torch")
    eng = ctd.Engine(0)
    try:
        # the walk first: the engine's prime and sieve buffers at full size
        walk = run(eng, 1)
        free, _ = torch.cuda.mem_get_info()
        room = 256 << 20
        assert room < 61 * MIN_PRIMES // 2
        filler = torch.empty(free - room, dtype=torch.uint8, device="cuda")
        try:
            assert torch.cuda.mem_get_info()[0] < 61 * MIN_PRIMES // 2
            auto = run(eng, 0)
        finally:
            del filler
            torch.cuda.empty_cache()
        assert auto.counts.tolist() == walk.counts.tolist()
        assert str(auto.to_factoring_results()) == str(walk.to_factoring_results())
        assert int(walk.counts.sum()) > 100
        # with room again the classified path runs and agrees
        again = run(eng, 0)
        assert str(again.to_factoring_results()) == str(walk.to_factoring_results())
    finally:
        eng.close()
