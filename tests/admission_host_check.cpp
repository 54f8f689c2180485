// Host-side check of the server's admission policy (ctd_admission.h, no
// CUDA).  Reads commands on stdin and prints the policy's state after each:
//   budget B max M        -- new policy
//   submit BYTES          -- queue a job of BYTES device bytes
//   fail K                -- the next K allocations fail
//   admit                 -- run admission; prints "rc admitted-ids"
//   release ID            -- the job ID finishes
// After every command: "used active queued".
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>

#include "../cutrialdive_gb300/csrc/ctd_admission.h"

struct Job {
    int id;
    uint64_t bytes;
};

int main()
{
    ctd::Admission<Job> adm;
    std::map<int, uint64_t> running;
    int next_id = 0, fail = 0;
    char cmd[32];
    while (std::scanf("%31s", cmd) == 1) {
        if (!std::strcmp(cmd, "budget")) {
            unsigned long long b;
            unsigned m;
            char kw[8];
            std::scanf("%llu %7s %u", &b, kw, &m);
            adm = ctd::Admission<Job>();
            adm.budget = b;
            adm.max_active = m;
            running.clear();
        } else if (!std::strcmp(cmd, "submit")) {
            unsigned long long b;
            std::scanf("%llu", &b);
            adm.queue.push_back(Job{next_id++, b});
        } else if (!std::strcmp(cmd, "fail")) {
            std::scanf("%d", &fail);
        } else if (!std::strcmp(cmd, "admit")) {
            std::string ids;
            const int rc = adm.admit([](const Job &j) { return j.bytes; },
                                     [&](Job &, uint64_t) { return fail > 0 ? (--fail, -3) : 0; },
                                     [&](Job &j) {
                                         running[j.id] = j.bytes;
                                         ids += " " + std::to_string(j.id);
                                     });
            std::printf("%d%s\n", rc, ids.c_str());
        } else if (!std::strcmp(cmd, "release")) {
            int id;
            std::scanf("%d", &id);
            adm.release(running[id]);
            running.erase(id);
        }
        std::printf("%llu %u %zu\n", (unsigned long long)adm.used, adm.active, adm.queue.size());
    }
    return 0;
}
