// Peel sequence of a pedigree: the elimination order of its members and, for
// each, the peel operation the samplers and the trait peel run.
//
// The operations follow the reference's PeelSequenceGenerator and
// PeelOperation (peel_sequence_generator.cc:57-250, peeling.h:17-339):
//   * the graph starts with every member adjacent to its parents, children
//     and mates (build_simple_graph); eliminating a member connects all of its
//     neighbours (eliminate_node);
//   * an operation's type is LAST if everyone else is peeled, CHILD if the
//     member has parents and neither is peeled, PARENT if the member has
//     children and neither all its mates nor all its children are peeled, else
//     PARTNER (set_type); a PARENT operation's children are the cutset members
//     that are its offspring, in cutset order;
//   * its previous functions are, repeatedly, the first unused earlier
//     operation whose cutset lies inside this cutset plus the peeled member
//     (find_prev_functions);
//   * an order is legal if no member is peeled while it could be both a CHILD
//     and a PARENT operation (is_legit).
// The order itself is found differently: the reference starts its randomised
// downhill search (exchanges of two random positions, get_cost = sum of cutset
// sizes) from a random permutation; here the search starts from a greedy
// minimum-cutset order (ties to the least fill-in, then the lowest index)
// among the members legal to peel next, its exchanges come from a fixed
// xorshift stream, and the cost is the rfunctions' work, sum of 4^|cutset|.
// Any legal order peels to the same likelihoods; the order changes only the
// work and the samplers' draw order.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/swiftlink_gb300.h"

namespace {

struct Op {
    int peel = 0;
    int type = 0;
    std::vector<int> cutset, prev, children;
};

enum { NULL_P = 0, CHILD_P = 1, PARENT_P = 2, PARTNER_P = 3, LAST_P = 4 };   // peeling.h:17-23

struct Ped {
    int n;
    std::vector<int> mo, fa;
    std::vector<std::vector<int>> children, mates;
    bool founder(int i) const { return mo[i] < 0; }
};

void add_node(std::vector<int>& v, int c) {
    if (std::find(v.begin(), v.end(), c) == v.end()) v.push_back(c);
}

void remove_node(std::vector<int>& v, int c) {
    auto it = std::find(v.begin(), v.end(), c);
    if (it != v.end()) v.erase(it);
}

std::vector<std::vector<int>> simple_graph(const Ped& p) {
    std::vector<std::vector<int>> g(p.n);
    for (int i = 0; i < p.n; ++i) {
        if (!p.founder(i)) {
            add_node(g[i], p.mo[i]);
            add_node(g[i], p.fa[i]);
        }
        for (int c : p.children[i]) add_node(g[i], c);
        for (int m : p.mates[i]) add_node(g[i], m);
    }
    return g;
}

void eliminate(std::vector<std::vector<int>>& g, int node) {
    const std::vector<int> cut = g[node];
    for (size_t i = 0; i < cut.size(); ++i) {
        remove_node(g[cut[i]], node);
        for (size_t j = 0; j < cut.size(); ++j)
            if (i != j) {
                add_node(g[cut[i]], cut[j]);
                add_node(g[cut[j]], cut[i]);
            }
    }
}

bool all_peeled(const std::vector<int>& v, const std::vector<char>& peeled) {
    for (int x : v)
        if (!peeled[x]) return false;
    return true;
}

// would peeling `i` now be both a CHILD and a PARENT operation (is_legit)
bool ambiguous(const Ped& p, int i, const std::vector<char>& peeled) {
    return !p.founder(i) && !(peeled[p.mo[i]] || peeled[p.fa[i]]) && !p.children[i].empty() &&
           !all_peeled(p.mates[i], peeled) && !all_peeled(p.children[i], peeled);
}

// cost of an order: the work of its rfunctions, sum of 4^|cutset| (get_proper_cost,
// peel_sequence_generator.cc:460-470), or -1 if the order is not legal
double order_cost(const Ped& p, const std::vector<int>& order) {
    auto g = simple_graph(p);
    std::vector<char> peeled(p.n, 0);
    double cost = 0.0;
    for (int node : order) {
        if (ambiguous(p, node, peeled)) return -1.0;
        cost += (double)(1ull << (2 * std::min<size_t>(g[node].size(), 30)));
        eliminate(g, node);
        peeled[node] = 1;
    }
    return cost;
}

// edges that eliminating `i` would add between its neighbours
int fill_in(const std::vector<std::vector<int>>& g, int i) {
    const std::vector<int>& c = g[i];
    int f = 0;
    for (size_t a = 0; a < c.size(); ++a)
        for (size_t b = a + 1; b < c.size(); ++b)
            if (std::find(g[c[a]].begin(), g[c[a]].end(), c[b]) == g[c[a]].end()) ++f;
    return f;
}

// greedy: the legal member with the smallest cutset, ties to the least fill-in,
// then to the lowest index
std::vector<int> greedy_order(const Ped& p) {
    auto g = simple_graph(p);
    std::vector<char> peeled(p.n, 0);
    std::vector<int> order;
    for (int step = 0; step < p.n; ++step) {
        int best = -1, best_fill = 0;
        for (int i = 0; i < p.n; ++i) {
            if (peeled[i] || ambiguous(p, i, peeled)) continue;
            if (best >= 0 && g[i].size() > g[best].size()) continue;
            const int f = fill_in(g, i);
            if (best < 0 || g[i].size() < g[best].size() || f < best_fill) {
                best = i;
                best_fill = f;
            }
        }
        if (best < 0)   // cannot happen: founders and leaves are never ambiguous
            for (int i = 0; i < p.n; ++i)
                if (!peeled[i]) { best = i; break; }
        order.push_back(best);
        eliminate(g, best);
        peeled[best] = 1;
    }
    return order;
}

// downhill search in the reference's manner (random_downhill_search,
// peel_sequence_generator.cc:350-409): exchange two random positions, keep the
// exchange when the order stays legal and its cost does not grow; a fixed
// xorshift stream makes the result reproducible
void downhill(const Ped& p, std::vector<int>& order, int iterations) {
    double cost = order_cost(p, order);
    uint64_t x = 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        return x;
    };
    const int n = (int)order.size();
    if (n < 2) return;
    for (int it = 0; it < iterations; ++it) {
        const int a = (int)(next() % (uint64_t)n);
        int b = (int)(next() % (uint64_t)n);
        if (a == b) continue;
        std::swap(order[a], order[b]);
        const double c = order_cost(p, order);
        if (c >= 0.0 && c <= cost) cost = c;
        else std::swap(order[a], order[b]);
    }
}

// finalise_peel_order (peel_sequence_generator.cc:227-245)
std::vector<Op> finalise(const Ped& p, const std::vector<int>& order) {
    auto g = simple_graph(p);
    std::vector<char> peeled(p.n, 0), used;
    std::vector<Op> ops;
    for (int node : order) {
        Op op;
        op.peel = node;
        op.cutset = g[node];
        // set_type (peel_sequence_generator.cc:188-222)
        bool last = true;
        for (int i = 0; i < p.n; ++i)
            if (i != node && !peeled[i]) last = false;
        if (last) op.type = LAST_P;
        else if (!p.founder(node) && !(peeled[p.mo[node]] || peeled[p.fa[node]])) op.type = CHILD_P;
        else if (!p.children[node].empty() && !all_peeled(p.mates[node], peeled) &&
                 !all_peeled(p.children[node], peeled))
            op.type = PARENT_P;
        else op.type = PARTNER_P;
        if (op.type == PARENT_P)
            for (int c : op.cutset)
                if (std::find(p.children[node].begin(), p.children[node].end(), c) != p.children[node].end())
                    op.children.push_back(c);
        // find_prev_functions (peel_sequence_generator.cc:57-83)
        std::vector<int> scope = op.cutset;
        scope.push_back(node);
        while (true) {
            int found = -1;
            for (size_t k = 0; k < ops.size(); ++k) {
                if (used[k]) continue;
                bool inside = true;
                for (int x : ops[k].cutset)
                    if (std::find(scope.begin(), scope.end(), x) == scope.end()) { inside = false; break; }
                if (inside) { found = (int)k; break; }
            }
            if (found < 0) break;
            used[found] = 1;
            op.prev.push_back(found);
        }
        eliminate(g, node);
        peeled[node] = 1;
        ops.push_back(op);
        used.push_back(0);
    }
    return ops;
}

}  // namespace

extern "C" int sl_peel_sequence(int32_t n, const int32_t* mother, const int32_t* father, int32_t capacity,
                                int32_t* op_type, int32_t* op_peelnode, int32_t* cutset_off, int32_t* cutset,
                                int32_t* prev_off, int32_t* prev, int32_t* children_off, int32_t* children) {
    if (n < 1 || !mother || !father || !op_type || !op_peelnode || !cutset_off || !cutset || !prev_off || !prev ||
        !children_off || !children)
        return SL_EINVAL;
    Ped p;
    p.n = n;
    p.mo.assign(mother, mother + n);
    p.fa.assign(father, father + n);
    p.children.assign(n, {});
    p.mates.assign(n, {});
    for (int i = 0; i < n; ++i) {
        if ((p.mo[i] < 0) != (p.fa[i] < 0) || p.mo[i] >= n || p.fa[i] >= n) return SL_EINVAL;
        if (p.mo[i] < 0) continue;
        // Person::add_child (person.cc:156-178): children in member order, mates once
        p.children[p.mo[i]].push_back(i);
        p.children[p.fa[i]].push_back(i);
        add_node(p.mates[p.mo[i]], p.fa[i]);
        add_node(p.mates[p.fa[i]], p.mo[i]);
    }
    std::vector<int> order = greedy_order(p);
    // the search costs O(n) per step: keep it to about 2 10^7 node visits
    downhill(p, order, std::max(200, std::min(20000, 20000000 / (n * n + 1))));
    if (order_cost(p, order) < 0.0) return SL_EINVAL;
    const std::vector<Op> ops = finalise(p, order);
    int32_t nc = 0, np = 0, nk = 0;
    cutset_off[0] = prev_off[0] = children_off[0] = 0;
    for (int k = 0; k < n; ++k) {
        const Op& op = ops[k];
        op_type[k] = op.type;
        op_peelnode[k] = op.peel;
        if (nc + (int32_t)op.cutset.size() > capacity || np + (int32_t)op.prev.size() > capacity ||
            nk + (int32_t)op.children.size() > capacity)
            return SL_ENOMEM;
        for (int x : op.cutset) cutset[nc++] = x;
        for (int x : op.prev) prev[np++] = x;
        for (int x : op.children) children[nk++] = x;
        cutset_off[k + 1] = nc;
        prev_off[k + 1] = np;
        children_off[k + 1] = nk;
    }
    return SL_OK;
}
