// Greedy RPA pair order against shared-memory bank collisions (see pair_order.hpp).
#include "pair_order.hpp"

#include <algorithm>
#include <map>

namespace spn {

namespace {

// Words read in one step, per (slot, phase, bank), at most 32 kept per bank.
class StepBanks {
public:
    explicit StepBanks(const PairBankModel &m) : m_(m), occ_(size_t(m.slots) * (32 / m.phase_lanes) * m.banks) {}
    // 1 if `word` would add a distinct word to an occupied bank
    int collides(int slot, int phase, int word) const {
        const std::vector<int> &o = occ_[index(slot, phase, word)];
        if (o.empty()) return 0;
        return std::find(o.begin(), o.end(), word) == o.end() ? 1 : 0;
    }
    void take(int slot, int phase, int word) {
        std::vector<int> &o = occ_[index(slot, phase, word)];
        if (std::find(o.begin(), o.end(), word) == o.end()) o.push_back(word);
    }
    long long extra() const {
        long long e = 0;
        for (const auto &o : occ_) e += o.empty() ? 0 : (long long)(o.size() - 1);
        return e;
    }

private:
    size_t index(int slot, int phase, int word) const {
        const int bank = ((word % m_.banks) + m_.banks) % m_.banks;
        return (size_t(slot) * (32 / m_.phase_lanes) + phase) * m_.banks + bank;
    }
    PairBankModel m_;
    std::vector<std::vector<int>> occ_;
};

}  // namespace

std::vector<int> order_pairs_by_banks(int n_sites, const int *ptr, const PairBankModel &m,
                                      const std::function<void(int, int *)> &words) {
    std::vector<int> out(static_cast<size_t>(ptr[n_sites]), 0);
    std::vector<int> w(m.slots);
    for (int g0 = 0; g0 < n_sites; g0 += 32) {
        const int g1 = std::min(n_sites, g0 + 32);
        std::vector<std::vector<int>> rem(g1 - g0);
        for (int j = g0; j < g1; ++j)
            for (int i = ptr[j]; i < ptr[j + 1]; ++i) rem[j - g0].push_back(i);
        std::vector<int> fill(g1 - g0, 0);
        for (;;) {
            bool any = false;
            StepBanks banks(m);
            for (int j = g0; j < g1; ++j) {
                std::vector<int> &cand = rem[j - g0];
                if (cand.empty()) continue;
                any = true;
                const int phase = (j - g0) / m.phase_lanes;
                size_t best = 0;
                int best_cost = 1 << 30;
                for (size_t q = 0; q < cand.size() && best_cost > 0; ++q) {
                    words(cand[q], w.data());
                    int cost = 0;
                    for (int s = 0; s < m.slots; ++s) cost += banks.collides(s, phase, w[s]);
                    if (cost < best_cost) {
                        best_cost = cost;
                        best = q;
                    }
                }
                const int i = cand[best];
                cand.erase(cand.begin() + long(best));
                words(i, w.data());
                for (int s = 0; s < m.slots; ++s) banks.take(s, phase, w[s]);
                out[size_t(ptr[j] + fill[j - g0]++)] = i;
            }
            if (!any) break;
        }
    }
    return out;
}

PairBankModel xyz_rpa_model() { return PairBankModel{2, 8, 8}; }

std::function<void(int, int *)> xyz_rpa_words(int nl, const int *rid1, const int *rid2, const int *perm1,
                                              const int *perm2) {
    return [=](int i, int *w) {
        w[0] = perm1[i] * nl + rid1[i];
        w[1] = 6 * nl + perm2[i] * nl + rid2[i];
    };
}

PairBankModel tri_rpa_model() { return PairBankModel{32, 32, 32}; }

std::function<void(int, int *)> tri_rpa_words(int nl, const int *rid1, const int *rid2, const int *perm1,
                                              const int *perm2) {
    // (X,Y,Z) (X,Z,Y) (Y,X,Z) (Y,Z,X) (Z,X,Y) (Z,Y,X); the density (3) maps to itself
    static const int perm[6][4] = {{0, 1, 2, 3}, {0, 2, 1, 3}, {1, 0, 2, 3}, {1, 2, 0, 3}, {2, 0, 1, 3}, {2, 1, 0, 3}};
    return [=](int i, int *w) {
        const int *p1 = perm[perm1[i]], *p2 = perm[perm2[i]];
        for (int c = 0; c < 16; ++c) {
            w[c] = (4 * p1[c >> 2] + p1[c & 3]) * nl + rid1[i];
            w[16 + c] = (4 * p2[c >> 2] + p2[c & 3]) * nl + rid2[i];
        }
    };
}

long long pair_bank_collisions(int n_sites, const int *ptr, const int *order, const PairBankModel &m,
                               const std::function<void(int, int *)> &words) {
    long long total = 0;
    std::vector<int> w(m.slots);
    for (int g0 = 0; g0 < n_sites; g0 += 32) {
        const int g1 = std::min(n_sites, g0 + 32);
        int steps = 0;
        for (int j = g0; j < g1; ++j) steps = std::max(steps, ptr[j + 1] - ptr[j]);
        for (int k = 0; k < steps; ++k) {
            StepBanks banks(m);
            for (int j = g0; j < g1; ++j) {
                if (k >= ptr[j + 1] - ptr[j]) continue;
                words(order[ptr[j] + k], w.data());
                for (int s = 0; s < m.slots; ++s) banks.take(s, (j - g0) / m.phase_lanes, w[s]);
            }
            total += banks.extra();
        }
    }
    return total;
}

}  // namespace spn
