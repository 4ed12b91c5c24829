// Planning of gpe_round_trip: which instances travel together (groups) and in
// which rounds each group steps (the rolling schedule).  Host-only C++ with no
// CUDA dependency, so that the CPU tests compile and check it directly.
#pragma once

#include <algorithm>
#include <vector>

namespace gpe {

constexpr int kRoundTripGroups = 4;

// Rounds [r0, r1) in which the same groups lo .. hi are active (lo > hi: none).
struct RoundTripPiece {
    long long r0, r1;
    int lo, hi;
};

struct RoundTripPlan {
    std::vector<std::vector<int>> groups;  // instance indices of each group
    std::vector<long long> join;           // the round in which each group takes its first step
    std::vector<RoundTripPiece> pieces;    // the rounds in order, cut where a group joins or leaves
};

// values[i]: values of instance i; order: the instances in work-item order
// (decreasing size); split: whether the instances may go in groups; steps: the
// K steps every instance takes; R: how many times longer one value takes to
// come over the host link than to take one step in HBM.
//
// Groups are contiguous runs of `order`, so that each group's work items are one
// contiguous range.  The first group holds half a share of the values and the
// others one share each (a group closes once the running count passes
// (g + 1/2) / (G - 1/2) of the total, if every later group still gets an
// instance): the steps wait for the first group's upload alone.  Without split
// (or without steps) there is one group, the instances in index order.
//
// A round advances every active group by one leapfrog step.  Group g is active
// in rounds join[g] .. join[g] + K - 1; groups join in order and leave in order.
// Group g + 1 joins once the rounds since group g joined have stepped about R
// times its values (its upload should have landed by then), and no later than
// the round after group g's last, so that no round is idle.
inline RoundTripPlan plan_round_trip(const std::vector<long long> &values, const std::vector<int> &order, bool split,
                                     long long steps, double R)
{
    RoundTripPlan p;
    const int n = int(values.size());
    if (!split || n < 2 || int(order.size()) != n || steps <= 0) {
        p.groups.emplace_back(n);
        for (int i = 0; i < n; i++) p.groups[0][i] = i;
    } else {
        const int G = std::min(n, kRoundTripGroups);
        long long total = 0;
        for (long long v : values) total += v;
        p.groups.resize(1);
        long long acc = 0;
        for (int k = 0; k < n; k++) {
            const int i = order[k];
            const int g = int(p.groups.size()) - 1;
            if (!p.groups[g].empty() && acc * (2 * G - 1) >= total * (2 * g + 1) && n - k >= G - g - 1 &&
                int(p.groups.size()) < G)
                p.groups.emplace_back();
            p.groups.back().push_back(i);
            acc += values[i];
        }
    }
    const int G = int(p.groups.size());
    p.join.assign(G, 0);
    std::vector<double> gv(G, 0.0);
    for (int g = 0; g < G; g++)
        for (int i : p.groups[g]) gv[g] += double(values[i]);
    for (int g = 0; g + 1 < G; g++) {
        double acc = 0.0;
        long long r = p.join[g];
        do {
            for (int q = 0; q <= g; q++)
                if (p.join[q] <= r && r < p.join[q] + steps) acc += gv[q];
            r++;
        } while (acc < R * gv[g + 1] && r < p.join[g] + steps);
        p.join[g + 1] = r;
    }
    std::vector<long long> cuts = {0};
    for (int g = 0; g < G; g++) {
        cuts.push_back(p.join[g]);
        cuts.push_back(p.join[g] + steps);
    }
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    for (size_t c = 0; c + 1 < cuts.size(); c++) {
        RoundTripPiece piece{cuts[c], cuts[c + 1], G, -1};
        for (int g = 0; g < G; g++)
            if (p.join[g] <= piece.r0 && piece.r0 < p.join[g] + steps) {
                piece.lo = std::min(piece.lo, g);
                piece.hi = std::max(piece.hi, g);
            }
        p.pieces.push_back(piece);
    }
    return p;
}

}  // namespace gpe
