// Prints the warp placement of schedule_groups (linear_system_solvers_gb300/csrc/heat1d_schedule.hpp)
// for the group costs read from standard input (one per line).
//   heat1d_schedule_t <sms> <warps_per_cta>
// Output: "ctas <c> warps_per_cta <w>", then one line per warp: its group indices.
#include "heat1d_schedule.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: heat1d_schedule_t <sms> <warps_per_cta> < costs\n");
        return 2;
    }
    const int sms = std::atoi(argv[1]), wpc = std::atoi(argv[2]);
    std::vector<double> work;
    double v;
    while (std::scanf("%lf", &v) == 1) work.push_back(v);
    const lss_gb300::heat1d::warp_schedule ws = lss_gb300::heat1d::schedule_groups(work, sms, wpc);
    std::printf("ctas %d warps_per_cta %d\n", ws.ctas, ws.warps_per_cta);
    const size_t nw = static_cast<size_t>(ws.ctas) * ws.warps_per_cta;
    for (size_t w = 0; w < nw; ++w) {
        for (int q = ws.first[w]; q < ws.first[w + 1]; ++q) std::printf(q == ws.first[w] ? "%d" : " %d", ws.group[q]);
        std::printf("\n");
    }
    return 0;
}
