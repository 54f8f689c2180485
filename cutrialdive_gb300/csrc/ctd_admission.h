// ctd_admission.h -- the server's admission policy (host only, no CUDA).
//
// Jobs wait in arrival order.  A job is admitted while fewer than
// `max_active` run and its device bytes fit the memory budget beside the
// jobs already running; a job larger than the whole budget is still
// admitted when nothing else runs, so it cannot wait forever.  Admission
// stops at the first job that does not fit (no overtaking: arrival order is
// kept).  The device allocation itself is the caller's `alloc(job, bytes)`;
// when it fails the job stays queued, the accounting is untouched, and the
// failure is returned, so a later call can retry once memory frees up.
//
// Kept free of CUDA so the policy and its failure paths are tested on the
// host with a fake allocator.
#pragma once

#include <cstdint>
#include <deque>

namespace ctd {

template <class Job>
struct Admission {
    uint64_t budget = 0;
    uint64_t used = 0;
    uint32_t max_active = 1;
    uint32_t active = 0;
    std::deque<Job> queue;

    bool fits(uint64_t bytes) const { return active == 0 || (used <= budget && bytes <= budget - used); }

    // Admits queued jobs in order.  bytes(job) gives a job's device bytes;
    // alloc(job, bytes) returns 0 on success or an error status, which
    // stops admission and is returned; admitted(job) takes the job.
    template <class Bytes, class Alloc, class Admitted>
    int admit(Bytes bytes, Alloc alloc, Admitted admitted)
    {
        while (!queue.empty() && active < max_active) {
            Job &j = queue.front();
            const uint64_t b = bytes(j);
            if (!fits(b))
                break;
            const int rc = alloc(j, b);
            if (rc)
                return rc;
            used += b;
            ++active;
            admitted(j);
            queue.pop_front();
        }
        return 0;
    }

    // a finished job gives back its bytes and its slot
    void release(uint64_t bytes)
    {
        used = bytes <= used ? used - bytes : 0;
        if (active)
            --active;
    }
};

}  // namespace ctd
