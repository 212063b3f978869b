// Drives the LP server's admission rule (acd-alm_gb300/csrc/admission.h) on
// scenarios read from stdin and prints its decisions, for
// tests/test_admission_host.py.
//
// Input, one scenario per line:
//   order <id nnz team> ...            -> prints the ids in admission order
//   pick sms busy budget in_use running backfill <id nnz team footprint waited> ...
//                                      -> prints the index picked (-1: none)
#include <algorithm>
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "admission.h"

int main()
{
        std::string line;
        while (std::getline(std::cin, line)) {
                std::istringstream in(line);
                std::string cmd;
                in >> cmd;
                std::vector<acd::Candidate> cs;
                if (cmd == "order") {
                        acd::Candidate c;
                        while (in >> c.id >> c.nnz >> c.team)
                                cs.push_back(c);
                        std::stable_sort(cs.begin(), cs.end(), acd::admits_before);
                        for (size_t i = 0; i < cs.size(); i++)
                                std::printf("%s%lld", i ? " " : "", cs[i].id);
                        std::printf("\n");
                } else if (cmd == "pick") {
                        acd::Capacity cap;
                        int running = 0;
                        in >> cap.sms >> cap.sms_busy >> cap.budget >> cap.in_use >> running
                           >> cap.backfill_seconds;
                        cap.nothing_running = running == 0;
                        acd::Candidate c;
                        while (in >> c.id >> c.nnz >> c.team >> c.footprint >> c.waited)
                                cs.push_back(c);
                        long at = acd::pick_admission(
                                cs.size(), [&](size_t i) { return cs[i]; }, cap);
                        std::printf("%ld\n", at);
                } else {
                        std::printf("?\n");
                }
        }
        return 0;
}
