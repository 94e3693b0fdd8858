// pow_sched.h -- schedules of polynomial products that compute X^e mod chi
// from byte-window tables (CUDA-free, shared by the library and its tests).
//
// The table of a characteristic polynomial holds, in slot 256 m + k, the
// polynomial X^(k * 2^(8 m)) mod chi for m < 8 and 0 < k < 256 (slots with
// k = 2^b are X^(2^(8 m + b)), made by squaring on the host).  Then
//   X^e = prod over the non-zero bytes e_m of e of slot(m, e_m),
// at most eight factors for a 64-bit exponent.  A schedule lists products
// (steps) level by level: the steps of one level are independent and run as
// one GPU launch, one CTA each; a step reads table slots or scratch slots
// written by earlier levels.
//   - serial: one step per exponent multiplies all its factors in turn;
//   - tree: the factors of an exponent are multiplied in pairs, level by
//     level (depth 3 for eight factors), so that a few exponents spread over
//     many CTAs.
// powSchedule picks the shape with fewer waves of `width` concurrent CTAs.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

namespace mtgp {

constexpr int kPowMaxSrc = 8;
constexpr int kPowSlots = 8 * 256;  // table slots per characteristic polynomial

inline int powSlot(int m, int k) { return m * 256 + k; }

// dst = product of src[0..nsrc) mod chi (nsrc = 0: the polynomial 1).
// src codes: >= 0 table slot, < 0 scratch slot -1 - code.  dst codes: >= 0
// output index (a table slot for table schedules), < 0 scratch slot.
// job: the exponent (or table) the step belongs to.
struct PowStep {
    int32_t job;
    int32_t nsrc;
    int32_t src[kPowMaxSrc];
    int32_t dst;
};

struct PowSchedule {
    std::vector<std::vector<PowStep>> levels;
    int nscratch = 0;
    int steps() const {
        int n = 0;
        for (const auto &l : levels) n += (int)l.size();
        return n;
    }
};

// The table factors of X^e: slots of the non-zero bytes, low byte first.
inline int powFactors(uint64_t e, int32_t *src) {
    int n = 0;
    for (int m = 0; m < 8; m++) {
        const int k = (int)((e >> (8 * m)) & 0xff);
        if (k) src[n++] = powSlot(m, k);
    }
    return n;
}

// Products filling the table: slot(m, k) = slot(m, k - low) * slot(m, low)
// with low the lowest set bit of k, by popcount of k (levels 0..6).
inline void tableSchedule(PowSchedule &s) {
    s.levels.assign(7, {});
    s.nscratch = 0;
    for (int m = 0; m < 8; m++)
        for (int k = 1; k < 256; k++) {
            const int pc = __builtin_popcount((unsigned)k);
            if (pc < 2) continue;
            PowStep st{};
            st.job = 0;
            st.nsrc = 2;
            st.src[0] = powSlot(m, k & (k - 1));
            st.src[1] = powSlot(m, k & -k);
            st.dst = powSlot(m, k);
            s.levels[(size_t)(pc - 2)].push_back(st);
        }
}

namespace pow_detail {
inline int64_t waves(int64_t n, int width) { return (n + width - 1) / width; }
}  // namespace pow_detail

// Steps computing X^e[j] into output j, j < n; width = CTAs that run at once.
inline void powSchedule(const uint64_t *e, int n, int width, PowSchedule &s) {
    s.levels.clear();
    s.nscratch = 0;
    if (n <= 0) return;
    if (width < 1) width = 1;
    std::vector<PowStep> base((size_t)n);
    int maxf = 0;
    for (int j = 0; j < n; j++) {
        PowStep &st = base[(size_t)j];
        st = PowStep{};
        st.job = j;
        st.nsrc = powFactors(e[j], st.src);
        st.dst = j;
        if (st.nsrc > maxf) maxf = st.nsrc;
    }
    // cost in products on the critical path: serial = the longer of the
    // longest chain and the products spread over the CTAs (the hardware
    // hands out CTAs as SMs free up); tree = sum over levels of the level's
    // waves (one product per step, a launch boundary between levels)
    std::vector<int64_t> per_level;
    for (int j = 0; j < n; j++) {
        int f = base[(size_t)j].nsrc;
        for (int l = 0; f > 1; l++) {
            if ((int)per_level.size() <= l) per_level.push_back(0);
            per_level[(size_t)l] += f / 2;
            f -= f / 2;
        }
    }
    int64_t tree_cost = 0;
    for (int64_t c : per_level) tree_cost += pow_detail::waves(c, width);
    int64_t products = 0;
    for (const PowStep &b : base) products += b.nsrc > 1 ? b.nsrc - 1 : 0;
    const int64_t serial_cost = std::max<int64_t>(maxf - 1, pow_detail::waves(products, width));
    if (maxf <= 2 || serial_cost <= tree_cost) {
        s.levels.push_back(std::move(base));
        return;
    }
    // tree: pair the factors; a leftover factor moves up unchanged
    std::vector<PowStep> first;  // exponents that need no product
    std::vector<std::vector<int32_t>> cur((size_t)n);
    for (int j = 0; j < n; j++) {
        const PowStep &b = base[(size_t)j];
        if (b.nsrc <= 1) {
            first.push_back(b);
        } else {
            cur[(size_t)j].assign(b.src, b.src + b.nsrc);
        }
    }
    s.levels.push_back(std::move(first));
    for (size_t l = 0;; l++) {
        if (s.levels.size() <= l) s.levels.emplace_back();
        bool any = false;
        for (int j = 0; j < n; j++) {
            std::vector<int32_t> &c = cur[(size_t)j];
            if (c.size() < 2) continue;
            any = true;
            std::vector<int32_t> next;
            const bool last = c.size() == 2;
            for (size_t q = 0; q + 1 < c.size(); q += 2) {
                PowStep st{};
                st.job = j;
                st.nsrc = 2;
                st.src[0] = c[q];
                st.src[1] = c[q + 1];
                if (last) {
                    st.dst = j;
                } else {
                    st.dst = -1 - s.nscratch++;
                    next.push_back(st.dst);
                }
                s.levels[l].push_back(st);
            }
            if (c.size() & 1) next.push_back(c.back());
            c = std::move(next);
        }
        if (!any) break;
    }
    while (!s.levels.empty() && s.levels.back().empty()) s.levels.pop_back();
}

}  // namespace mtgp
