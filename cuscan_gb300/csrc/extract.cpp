// Host-side cluster extraction from a finished MST (no device work).
//
// Restates hdbscan_core::clusters_from_spanning_tree (crates/hdbscan-core/src/lib.rs:57-97)
// and the stages it calls, in the same order and with the same tie and float rules:
//   sort_mst / mst_to_linkage        crates/hdbscan-core/src/linkage.rs:25-101
//   condense_tree                    crates/hdbscan-core/src/condense.rs:87-156
//   simplify_hierarchy               crates/hdbscan-core/src/condense.rs:162-262
//   select_clusters (EOM/leaf/eps)   crates/hdbscan-core/src/select.rs:10-227
//   argsort (Numba quicksort order)  crates/hdbscan-core/src/argsort.rs:3-80
//   labels / membership strengths    crates/hdbscan-core/src/labels.rs:14-151
//   dbscan_cut                       crates/hdbscan-core/src/labels.rs:154-209
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <new>
#include <set>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "cuscan_gb300.h"

namespace {

struct SortedEdge {
    uint32_t src, dst;
    double w;
};

struct LinkageRow {
    size_t left, right;
    double distance;
    size_t size;
};

struct Condensed {
    std::vector<size_t> parent, child;
    std::vector<float> lambda, child_size;
    size_t size() const { return parent.size(); }
    bool empty() const { return parent.empty(); }
    void push(size_t p, size_t c, float l, float s) {
        parent.push_back(p);
        child.push_back(c);
        lambda.push_back(l);
        child_size.push_back(s);
    }
    Condensed cluster_tree() const {
        Condensed out;
        for (size_t i = 0; i < size(); ++i)
            if (child_size[i] > 1.0f) out.push(parent[i], child[i], lambda[i], child_size[i]);
        return out;
    }
};

struct Error : std::runtime_error {
    int kind;
    Error(int k, const std::string &m) : std::runtime_error(m), kind(k) {}
};

// Rank DSU, first argument wins ties, path halving (crates/hdbscan-core/src/dsu.rs).
struct RankDsu {
    std::vector<size_t> parent;
    std::vector<uint32_t> rank;
    explicit RankDsu(size_t n) : parent(n), rank(n, 0) {
        for (size_t i = 0; i < n; ++i) parent[i] = i;
    }
    size_t find(size_t x) {
        while (parent[x] != x) {
            size_t p = parent[x];
            parent[x] = parent[p];
            x = p;
        }
        return x;
    }
    void union_roots(size_t x, size_t y) {
        if (x == y) return;
        if (rank[x] < rank[y]) std::swap(x, y);
        parent[y] = x;
        if (rank[x] == rank[y]) rank[x] += 1;
    }
    void unite(size_t x, size_t y) { union_roots(find(x), find(y)); }
};

// f64::total_cmp as a signed 64-bit key.
inline int64_t total_key(double x) {
    int64_t b;
    std::memcpy(&b, &x, 8);
    return b ^ (int64_t)(((uint64_t)(b >> 63)) >> 1);
}

void sort_mst(std::vector<SortedEdge> &edges) {
    for (auto &e : edges)
        if (e.w == 0.0) e.w = 0.0;
    std::sort(edges.begin(), edges.end(), [](const SortedEdge &a, const SortedEdge &b) {
        int64_t ka = total_key(a.w), kb = total_key(b.w);
        if (ka != kb) return ka < kb;
        if (a.src != b.src) return a.src < b.src;
        return a.dst < b.dst;
    });
}

std::vector<LinkageRow> mst_to_linkage(const std::vector<SortedEdge> &edges) {
    const size_t n = edges.size() + 1;
    const size_t slots = 2 * n - 1;
    std::vector<size_t> parent(slots), size(slots, 0);
    for (size_t i = 0; i < slots; ++i) parent[i] = i;
    for (size_t i = 0; i < n; ++i) size[i] = 1;
    auto find = [&](size_t x) {
        while (parent[x] != x) {
            size_t p = parent[x];
            parent[x] = parent[p];
            x = p;
        }
        return x;
    };
    std::vector<LinkageRow> rows;
    rows.reserve(edges.size());
    for (size_t index = 0; index < edges.size(); ++index) {
        const auto &e = edges[index];
        if (e.src >= n || e.dst >= n)
            throw Error(CUSCAN_INVALID_INPUT,
                        "MST edge " + std::to_string(index) + " endpoint is out of range for " +
                            std::to_string(n) + " points");
        if (std::isnan(e.w) || e.w < 0.0)
            throw Error(CUSCAN_INVALID_INPUT, "MST edge " + std::to_string(index) +
                                                  " weight must be nonnegative and not NaN");
        size_t left = find(e.src), right = find(e.dst);
        if (left == right)
            throw Error(CUSCAN_INVALID_INPUT, "MST edge " + std::to_string(index) + " closes a cycle");
        size_t big = left > right ? left : right, small = left > right ? right : left;
        size_t next = n + index;
        size[next] = size[left] + size[right];
        parent[left] = next;
        parent[right] = next;
        rows.push_back({big, small, e.w, size[next]});
    }
    return rows;
}

float lambda_value(double distance) {
    return distance > 0.0 ? (float)(1.0 / distance) : std::numeric_limits<float>::infinity();
}

std::vector<size_t> bfs_from_hierarchy(const std::vector<LinkageRow> &h, size_t root, size_t np) {
    std::vector<size_t> result{root};
    size_t start = 0;
    while (start < result.size()) {
        size_t end = result.size();
        for (size_t pos = start; pos < end; ++pos) {
            size_t node = result[pos];
            if (node >= np) {
                const auto &row = h[node - np];
                result.push_back(row.left);
                result.push_back(row.right);
            }
        }
        start = end;
    }
    return result;
}

Condensed condense_tree(const std::vector<LinkageRow> &h, size_t min_cluster_size) {
    Condensed tree;
    if (h.empty()) return tree;
    const size_t np = h.size() + 1;
    const size_t root = 2 * h.size();
    const double min_size = (double)min_cluster_size;
    size_t next_label = np + 1;
    std::vector<size_t> relabel(root + 1, 0);
    relabel[root] = np;
    std::vector<char> ignore(root + 1, 0);
    auto count = [&](size_t node) -> float { return node >= np ? (float)h[node - np].size : 1.0f; };
    auto eliminate = [&](size_t branch, size_t parent, float lambda) {
        if (branch < np) {
            tree.push(parent, branch, lambda, 1.0f);
        } else {
            for (size_t sub : bfs_from_hierarchy(h, branch, np)) {
                if (sub < np)
                    tree.push(parent, sub, lambda, 1.0f);
                else
                    ignore[sub] = 1;
            }
        }
    };
    for (size_t node : bfs_from_hierarchy(h, root, np)) {
        if (ignore[node] || node < np) continue;
        size_t parent = relabel[node];
        const LinkageRow row = h[node - np];
        size_t left = row.left, right = row.right;
        float lambda = lambda_value(row.distance);
        float lc = count(left), rc = count(right);
        bool left_small = (double)lc < min_size;
        bool right_small = (double)rc < min_size;
        if (left < np && !right_small) {
            relabel[right] = parent;
            tree.push(parent, left, lambda, 1.0f);
        } else if (left_small && !right_small) {
            relabel[right] = parent;
            eliminate(left, parent, lambda);
        } else if (!left_small && right_small) {
            relabel[left] = parent;
            eliminate(right, parent, lambda);
        } else if (left_small && right_small) {
            eliminate(left, parent, lambda);
            eliminate(right, parent, lambda);
        } else {
            relabel[left] = next_label;
            tree.push(parent, next_label, lambda, lc);
            ++next_label;
            relabel[right] = next_label;
            tree.push(parent, next_label, lambda, rc);
            ++next_label;
        }
    }
    return tree;
}

Condensed simplify_hierarchy(const Condensed &tree, double threshold) {
    Condensed ct = tree.cluster_tree();
    if (tree.empty() || ct.empty()) return tree;
    const size_t np = tree.parent[0];
    const size_t n_nodes = ct.child[ct.size() - 1] + 1;
    const size_t width = n_nodes - np;
    std::vector<char> leaf(width, 1);
    for (size_t p : ct.parent) leaf[p - np] = 0;
    std::vector<float> max_births(width, 0.0f);
    for (size_t i = 0; i < tree.size(); ++i) max_births[tree.parent[i] - np] = tree.lambda[i];
    std::vector<size_t> parent_map(width);
    for (size_t i = 0; i < width; ++i) parent_map[i] = np + i;
    std::unordered_map<size_t, float> lambda_map;
    size_t idx = ct.size() - 1;
    while (idx > 0) {
        size_t parent = ct.parent[idx];
        size_t children[2] = {ct.child[idx - 1], ct.child[idx]};
        float death = ct.lambda[idx];
        size_t nodes[2] = {children[0] - np, children[1] - np};
        float births[2] = {max_births[nodes[0]], max_births[nodes[1]]};
        float birth_max = births[1] > births[0] ? births[1] : births[0];
        float birth_min = births[1] < births[0] ? births[1] : births[0];
        size_t slot = parent - np;
        if (birth_max > max_births[slot]) max_births[slot] = birth_max;
        double persistence = (double)(birth_min - death);
        // upstream keeps the split when persistence >= threshold; NaN is simplified
        if (!(persistence >= threshold)) {
            size_t sibling = births[0] <= births[1] ? 1 : 0;
            if (leaf[nodes[sibling]]) {
                leaf[slot] = 1;
            } else {
                lambda_map[children[1 - sibling]] = death;
            }
            parent_map[nodes[0]] = parent;
            parent_map[nodes[1]] = parent;
        }
        if (idx < 2) break;
        idx -= 2;
    }
    for (size_t i = 0; i < width; ++i) parent_map[i] = parent_map[parent_map[i] - np];
    std::vector<char> skipped(width, 0);
    std::vector<size_t> prefix(width + 1, 0);
    for (size_t i = 0; i < width; ++i) {
        size_t parent = parent_map[i];
        skipped[i] = parent != i + np;
        prefix[i + 1] = prefix[i] + (skipped[i] ? 1 : 0);
        parent_map[i] = parent - prefix[parent - np];
    }
    Condensed out;
    for (size_t index = 0; index < tree.size(); ++index) {
        size_t parent = tree.parent[index], child = tree.child[index];
        size_t cidx = child >= np ? child - np : 0;
        if (skipped[cidx]) continue;
        auto it = lambda_map.find(parent);
        float lambda = it != lambda_map.end() ? it->second : tree.lambda[index];
        size_t c = child >= np ? parent_map[child - np] : child;
        out.push(parent_map[parent - np], c, lambda, tree.child_size[index]);
    }
    return out;
}

// Numba quicksort permutation (crates/hdbscan-core/src/argsort.rs).
std::vector<size_t> numba_argsort(const std::vector<size_t> &values) {
    const size_t SMALL = 15;
    std::vector<size_t> order(values.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    if (order.size() < 2) return order;
    std::vector<std::pair<size_t, size_t>> stack(100);
    stack[0] = {0, order.size() - 1};
    size_t depth = 1;
    while (depth > 0) {
        --depth;
        size_t low = stack[depth].first, high = stack[depth].second;
        while (high - low >= SMALL) {
            size_t mid = (low + high) >> 1;
            if (values[order[mid]] < values[order[low]]) std::swap(order[low], order[mid]);
            if (values[order[high]] < values[order[mid]]) std::swap(order[high], order[mid]);
            if (values[order[mid]] < values[order[low]]) std::swap(order[low], order[mid]);
            size_t pivot = values[order[mid]];
            std::swap(order[high], order[mid]);
            // signed cursors: j may step below `low`
            int64_t i = (int64_t)low, j = (int64_t)high - 1;
            for (;;) {
                while (i < (int64_t)high && values[order[i]] < pivot) ++i;
                while (j >= (int64_t)low && pivot < values[order[j]]) --j;
                if (i >= j) break;
                std::swap(order[i], order[j]);
                ++i;
                --j;
            }
            std::swap(order[i], order[high]);
            size_t ui = (size_t)i;
            if (high - ui > ui - low) {
                if (high > ui) {
                    if (depth >= stack.size()) stack.resize(stack.size() * 2);
                    stack[depth++] = {ui + 1, high};
                }
                if (ui == low) {
                    low = high;
                    break;
                }
                high = ui - 1;
            } else {
                if (ui > low) {
                    if (depth >= stack.size()) stack.resize(stack.size() * 2);
                    stack[depth++] = {low, ui - 1};
                }
                if (ui == high) {
                    low = high;
                    break;
                }
                low = ui + 1;
            }
        }
        for (size_t i = low + 1; i <= high && low < high + 1; ++i) {
            if (i > high) break;
            size_t key = order[i];
            size_t j = i;
            while (j > low && values[key] < values[order[j - 1]]) {
                order[j] = order[j - 1];
                --j;
            }
            order[j] = key;
        }
    }
    return order;
}

std::vector<size_t> extract_eom(const Condensed &condensed, const Condensed &tree, size_t np,
                                int64_t max_size, bool allow_root) {
    if (tree.empty()) return {};
    size_t maxid = 0;
    for (size_t c : tree.child) maxid = std::max(maxid, c);
    for (size_t p : tree.parent) maxid = std::max(maxid, p);
    const size_t width = maxid - np + 1;
    std::vector<float> scores(width, 0.0f), sizes(width, 0.0f);
    std::vector<std::vector<size_t>> children(width);
    std::vector<char> born(width, 0);
    born[0] = 1;
    const size_t root = np;
    sizes[0] = (float)(np > 0 ? np - 1 : 0);
    std::vector<size_t> insertion_order{root};
    for (size_t i = 0; i < condensed.size(); ++i) {
        size_t parent = condensed.parent[i], child = condensed.child[i];
        float score = condensed.lambda[i] * condensed.child_size[i];
        size_t pi = parent - np;
        if (condensed.child_size[i] > 1.0f) {
            size_t ci = child - np;
            scores[ci] = -score;
            sizes[ci] = condensed.child_size[i];
            if (!born[ci]) insertion_order.push_back(child);
            born[ci] = 1;
            children[pi].push_back(child);
        }
        scores[pi] += score;
    }
    std::vector<size_t> roots = allow_root ? std::vector<size_t>{root} : children[0];
    std::vector<char> chosen(width, 0);
    std::vector<double> value(width, 0.0);
    for (size_t start : roots) {
        std::vector<std::pair<size_t, bool>> stack{{start, false}};
        while (!stack.empty()) {
            auto [node, visited] = stack.back();
            stack.pop_back();
            size_t index = node - np;
            if (!visited) {
                stack.push_back({node, true});
                for (auto it = children[index].rbegin(); it != children[index].rend(); ++it)
                    stack.push_back({*it, false});
            } else {
                double child_total = 0.0;
                for (size_t c : children[index]) child_total += value[c - np];
                double current = (double)(0.0f > scores[index] ? 0.0f : scores[index]);
                bool too_large = max_size > 0 && (double)sizes[index] > (double)max_size;
                if (child_total > current || too_large) {
                    value[index] = child_total;
                } else {
                    chosen[index] = 1;
                    value[index] = current;
                }
            }
        }
    }
    std::vector<char> selected(width, 0);
    std::vector<std::pair<size_t, bool>> stack;
    for (auto it = roots.rbegin(); it != roots.rend(); ++it) stack.push_back({*it, false});
    while (!stack.empty()) {
        auto [node, anc] = stack.back();
        stack.pop_back();
        size_t index = node - np;
        bool here = !anc && chosen[index];
        selected[index] = here;
        for (auto it = children[index].rbegin(); it != children[index].rend(); ++it)
            stack.push_back({*it, anc || here});
    }
    std::vector<size_t> out;
    for (size_t node : insertion_order)
        if (selected[node - np]) out.push_back(node);
    return out;
}

std::vector<size_t> leaves(const Condensed &tree) {
    if (tree.empty()) return {};
    std::unordered_set<size_t> parents(tree.parent.begin(), tree.parent.end());
    std::vector<size_t> result;
    for (size_t c : tree.child)
        if (!parents.count(c)) result.push_back(c);
    std::sort(result.begin(), result.end());
    return result;
}

size_t partition_point_child(const std::vector<size_t> &child, size_t value) {
    return (size_t)(std::lower_bound(child.begin(), child.end(), value) - child.begin());
}

size_t traverse_upwards(size_t node, double epsilon, size_t root, const Condensed &tree) {
    size_t segment = node;
    for (;;) {
        auto it = std::find(tree.child.begin(), tree.child.end(), segment);
        if (it == tree.child.end()) return root;
        size_t parent = tree.parent[(size_t)(it - tree.child.begin())];
        if (parent == root) return root;
        size_t idx = partition_point_child(tree.child, parent);
        float lambda = idx < tree.lambda.size() ? tree.lambda[idx] : 0.0f;
        double death_eps = lambda > 0.0f ? 1.0 / (double)lambda
                                         : std::numeric_limits<double>::infinity();
        if (death_eps >= epsilon) return parent;
        segment = parent;
    }
}

std::unordered_set<size_t> segments_in_branch(size_t segment, const std::vector<size_t> &parents,
                                              const std::vector<size_t> &children) {
    std::unordered_set<size_t> result;
    std::vector<size_t> pending{segment};
    while (!pending.empty()) {
        std::vector<size_t> next;
        for (size_t node : pending) {
            if (!result.insert(node).second) continue;
            size_t idx = (size_t)(std::lower_bound(parents.begin(), parents.end(), node) -
                                  parents.begin());
            if (idx < parents.size()) {
                next.push_back(children[idx]);
                if (idx + 1 < children.size()) next.push_back(children[idx + 1]);
            }
        }
        pending.swap(next);
    }
    return result;
}

std::vector<size_t> epsilon_search(const std::vector<size_t> &selected, const Condensed &tree,
                                   double epsilon) {
    std::vector<size_t> order = numba_argsort(tree.parent);
    std::vector<size_t> parents(order.size()), children(order.size());
    for (size_t i = 0; i < order.size(); ++i) {
        parents[i] = tree.parent[order[i]];
        children[i] = tree.child[order[i]];
    }
    size_t root = *std::min_element(tree.parent.begin(), tree.parent.end());
    std::unordered_set<size_t> processed;
    std::vector<size_t> output;
    for (size_t cluster : selected) {
        size_t idx = partition_point_child(tree.child, cluster);
        float lambda = idx < tree.lambda.size() ? tree.lambda[idx] : 0.0f;
        double death_eps =
            lambda > 0.0f ? 1.0 / (double)lambda : std::numeric_limits<double>::infinity();
        if (death_eps < epsilon) {
            if (!processed.count(cluster)) {
                size_t ancestor = traverse_upwards(cluster, epsilon, root, tree);
                output.push_back(ancestor);
                auto seg = segments_in_branch(ancestor, parents, children);
                processed.insert(seg.begin(), seg.end());
            }
        } else {
            output.push_back(cluster);
        }
    }
    return output;
}

std::vector<size_t> select_clusters(const Condensed &tree, size_t np,
                                    const cuscan_extract_config &cfg) {
    Condensed ct = tree.cluster_tree();
    std::vector<size_t> selected =
        cfg.selection_leaf ? leaves(ct)
                           : extract_eom(tree, ct, np, cfg.max_cluster_size,
                                         cfg.allow_single_cluster != 0);
    if (selected.size() > 1 && cfg.cluster_selection_epsilon > 0.0)
        selected = epsilon_search(selected, ct, cfg.cluster_selection_epsilon);
    return selected;
}

std::vector<int32_t> get_cluster_label_vector(const Condensed &tree,
                                              const std::vector<size_t> &clusters, double eps,
                                              size_t np) {
    std::vector<int32_t> labels(np, -1);
    if (tree.empty() || clusters.empty() || np == 0) return labels;
    std::vector<size_t> sorted = clusters;
    std::sort(sorted.begin(), sorted.end());
    std::unordered_map<size_t, int32_t> label_map;
    for (size_t i = 0; i < sorted.size(); ++i) label_map[sorted[i]] = (int32_t)i;
    size_t maxid = 0;
    for (size_t v : tree.parent) maxid = std::max(maxid, v);
    for (size_t v : tree.child) maxid = std::max(maxid, v);
    std::vector<char> selected(maxid + 1, 0);
    for (size_t c : clusters)
        if (c < selected.size()) selected[c] = 1;
    const size_t slots = std::max(maxid, np > 0 ? np - 1 : 0) + 1;
    RankDsu dsu(slots);
    std::vector<float> point_lambda(np, 0.0f);
    float root_max_lambda = 0.0f;
    const size_t root = np;
    for (size_t i = 0; i < tree.size(); ++i) {
        size_t parent = tree.parent[i], child = tree.child[i];
        float lambda = tree.lambda[i];
        if (parent == root) root_max_lambda = std::fmax(root_max_lambda, lambda);
        if (child < np) point_lambda[child] = lambda;
        bool sel = child < selected.size() ? selected[child] != 0 : false;
        if (!sel) {
            if (child < np && lambda == 0.0f) continue;
            if (parent < slots && child < slots) dsu.unite(parent, child);
        }
    }
    std::set<size_t> distinct(clusters.begin(), clusters.end());
    bool single_root = distinct.size() == 1 && clusters[0] == root;
    for (size_t point = 0; point < np; ++point) {
        size_t rep = dsu.find(point);
        if (rep < root) continue;
        if (rep == root) {
            if (single_root) {
                double lambda = (double)point_lambda[point];
                bool include = eps > 0.0 ? lambda >= 1.0 / eps : lambda >= (double)root_max_lambda;
                if (include) {
                    auto it = label_map.find(root);
                    labels[point] = it != label_map.end() ? it->second : -1;
                }
            }
        } else {
            auto it = label_map.find(rep);
            labels[point] = it != label_map.end() ? it->second : -1;
        }
    }
    return labels;
}

std::vector<float> membership_strengths(const Condensed &tree, const std::vector<size_t> &sel_sorted,
                                        const std::vector<int32_t> &labels, size_t np) {
    std::vector<float> out(labels.size(), 0.0f);
    if (tree.empty() || sel_sorted.empty()) return out;
    std::unordered_map<size_t, double> max_lambdas;
    for (size_t i = 0; i < tree.size(); ++i) {
        if (tree.child_size[i] == 1.0f &&
            std::binary_search(sel_sorted.begin(), sel_sorted.end(), tree.parent[i])) {
            double lambda = (double)tree.lambda[i];
            double &m = max_lambdas[tree.parent[i]];  // default 0.0
            m = std::fmax(m, lambda);
        }
    }
    for (size_t i = 0; i < tree.size(); ++i) {
        size_t point = tree.child[i];
        if (point >= np || point >= labels.size() || labels[point] < 0) continue;
        size_t cl = (size_t)labels[point];
        if (cl >= sel_sorted.size()) continue;
        size_t cluster = sel_sorted[cl];
        auto it = max_lambdas.find(cluster);
        double maximum = it != max_lambdas.end() ? it->second : 0.0;
        float lambda = tree.lambda[i];
        out[point] = (maximum == 0.0 || !std::isfinite(lambda))
                         ? 1.0f
                         : (float)(std::fmin((double)lambda, maximum) / maximum);
    }
    return out;
}

}  // namespace

struct cuscan_clustering {
    std::vector<int32_t> labels;
    std::vector<float> probabilities;
    std::vector<LinkageRow> linkage;
    Condensed condensed;
    std::vector<SortedEdge> sorted_mst;
};

extern "C" {

static void set_err(char *err, size_t len, const char *msg) {
    if (err && len) {
        std::strncpy(err, msg, len - 1);
        err[len - 1] = 0;
    }
}

int cuscan_clusters_from_spanning_tree(const uint32_t *src, const uint32_t *dst,
                                       const double *weight, int64_t m,
                                       const cuscan_extract_config *config,
                                       cuscan_clustering **out, char *err, size_t err_len) {
    if (!out || !config) {
        set_err(err, err_len, "null argument");
        return CUSCAN_INVALID_INPUT;
    }
    *out = nullptr;
    if (config->min_cluster_size <= 0) {
        set_err(err, err_len, "min_cluster_size must be positive");
        return CUSCAN_INVALID_CONFIG;
    }
    for (double v : {config->cluster_selection_epsilon, config->cluster_selection_persistence}) {
        if (!std::isfinite(v) || v < 0.0) {
            set_err(err, err_len, "cluster selection thresholds must be finite and non-negative");
            return CUSCAN_INVALID_CONFIG;
        }
    }
    if (m < 0 || (m > 0 && (!src || !dst || !weight))) {
        set_err(err, err_len, "invalid MST arrays");
        return CUSCAN_INVALID_INPUT;
    }
    if (m + 1 > (int64_t)INT32_MAX) {
        set_err(err, err_len, "point index exceeds the supported integer range");
        return CUSCAN_OVERFLOW;
    }
    try {
        auto *r = new cuscan_clustering();
        if (m == 0) {  // one finite row: all noise, empty trees (lib.rs:40-50)
            r->labels = {-1};
            r->probabilities = {0.0f};
            *out = r;
            return CUSCAN_OK;
        }
        const size_t np = (size_t)m + 1;
        r->sorted_mst.resize((size_t)m);
        for (int64_t i = 0; i < m; ++i) r->sorted_mst[i] = {src[i], dst[i], weight[i]};
        sort_mst(r->sorted_mst);
        r->linkage = mst_to_linkage(r->sorted_mst);
        r->condensed = condense_tree(r->linkage, (size_t)config->min_cluster_size);
        if (config->cluster_selection_persistence > 0.0 && !r->condensed.empty())
            r->condensed = simplify_hierarchy(r->condensed, config->cluster_selection_persistence);
        std::vector<size_t> selected = select_clusters(r->condensed, np, *config);
        r->labels = get_cluster_label_vector(r->condensed, selected,
                                             config->cluster_selection_epsilon, np);
        std::vector<size_t> sorted = selected;
        std::sort(sorted.begin(), sorted.end());
        r->probabilities = membership_strengths(r->condensed, sorted, r->labels, np);
        *out = r;
        return CUSCAN_OK;
    } catch (const Error &e) {
        set_err(err, err_len, e.what());
        return e.kind;
    } catch (const std::bad_alloc &) {
        set_err(err, err_len, "host allocation failed during cluster extraction");
        return CUSCAN_MEMORY;
    }
}

int64_t cuscan_clustering_points(const cuscan_clustering *r) {
    return r ? (int64_t)r->labels.size() : 0;
}

int64_t cuscan_clustering_condensed_rows(const cuscan_clustering *r) {
    return r ? (int64_t)r->condensed.size() : 0;
}

void cuscan_clustering_read(const cuscan_clustering *r, int32_t *labels, float *probabilities,
                            double *linkage, double *sorted_mst, int64_t *condensed_parent,
                            int64_t *condensed_child, float *condensed_lambda,
                            float *condensed_child_size) {
    if (!r) return;
    if (labels) std::memcpy(labels, r->labels.data(), r->labels.size() * sizeof(int32_t));
    if (probabilities)
        std::memcpy(probabilities, r->probabilities.data(), r->probabilities.size() * sizeof(float));
    if (linkage)
        for (size_t i = 0; i < r->linkage.size(); ++i) {
            linkage[4 * i + 0] = (double)r->linkage[i].left;
            linkage[4 * i + 1] = (double)r->linkage[i].right;
            linkage[4 * i + 2] = r->linkage[i].distance;
            linkage[4 * i + 3] = (double)r->linkage[i].size;
        }
    if (sorted_mst)
        for (size_t i = 0; i < r->sorted_mst.size(); ++i) {
            sorted_mst[3 * i + 0] = (double)r->sorted_mst[i].src;
            sorted_mst[3 * i + 1] = (double)r->sorted_mst[i].dst;
            sorted_mst[3 * i + 2] = r->sorted_mst[i].w;
        }
    for (size_t i = 0; i < r->condensed.size(); ++i) {
        if (condensed_parent) condensed_parent[i] = (int64_t)r->condensed.parent[i];
        if (condensed_child) condensed_child[i] = (int64_t)r->condensed.child[i];
        if (condensed_lambda) condensed_lambda[i] = r->condensed.lambda[i];
        if (condensed_child_size) condensed_child_size[i] = r->condensed.child_size[i];
    }
}

void cuscan_clustering_free(cuscan_clustering *r) { delete r; }

// DBSCAN labels at a strict single-linkage cut (crates/hdbscan-core/src/labels.rs:154-209).
// linkage is [rows*4] (left, right, distance, size); labels_out has rows+1 entries.
int cuscan_dbscan_cut(const double *linkage, int64_t rows, double cut, int64_t min_size,
                      int32_t *labels_out) {
    if (std::isnan(cut)) return CUSCAN_INVALID_CONFIG;
    const size_t np = (size_t)rows + 1;
    const size_t slots = 2 * (size_t)rows + 1;
    RankDsu dsu(slots);
    for (int64_t index = 0; index < rows; ++index) {
        double dist = linkage[4 * index + 2];
        if (dist < cut) {
            size_t cluster = np + (size_t)index;
            size_t left = (size_t)linkage[4 * index], right = (size_t)linkage[4 * index + 1];
            if (left >= slots || right >= slots) return CUSCAN_INVALID_INPUT;
            dsu.unite(left, cluster);
            dsu.unite(right, cluster);
        }
    }
    std::vector<size_t> reps(np);
    std::map<size_t, size_t> sizes;
    for (size_t p = 0; p < np; ++p) {
        reps[p] = dsu.find(p);
        sizes[reps[p]] += 1;
    }
    std::unordered_map<size_t, int32_t> label_map;
    int32_t next = 0;
    for (auto &kv : sizes) label_map[kv.first] = kv.second < (size_t)min_size ? -1 : next++;
    for (size_t p = 0; p < np; ++p) labels_out[p] = label_map[reps[p]];
    return CUSCAN_OK;
}

}  // extern "C"
