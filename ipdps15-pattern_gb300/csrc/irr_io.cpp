// irr_io.cpp -- the drivers' graph and coordinate file formats (host code).
//
// Graph (moldyn/misc.c:62-146, ReadInputGraph): lines starting with '%' before
// the header are skipped; the header is "<nodes> <edges>"; then one line per
// node i (1-based ids) listing its neighbours.  A line is read up to its first
// value <= 0 or non-number, and only neighbours j >= i are kept, so each
// undirected pair is listed once (as (i, j) with i <= j) and the header's edge
// count must equal the number kept.  moldyn's misc.c defines CSTYLE
// (misc.c:20), so its reader returns 0-based pairs [0, n), which is the
// default here (the library's node ids); `one_based` gives the [1, n] pairs of
// its non-CSTYLE branch.  A node line missing at the end of the file counts as
// empty, as in the reference.  Differences, on files the reference does not
// read: a last line without its newline is read here (the reference stops at
// end of file before parsing it), and lines are not limited to its 1,280,000
// characters.
// Coordinates (moldyn/misc.c:224-246, ReadCoord): whitespace-separated x y z
// triples, exactly num_nodes of them (reading stops at the first token that is
// not a number, where the reference's fscanf loop would not end).
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/irregular_gb300.h"

extern "C" {

int irr_read_graph(const char* path, int64_t* num_nodes, int64_t* num_edges, int32_t* edges,
                   int64_t cap, int one_based)
{
    if (!path || !num_nodes || !num_edges) return IRR_ERR_ARG;
    std::ifstream in(path);
    if (!in) return IRR_ERR_ARG;
    std::string line;
    bool have_header = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line[0] == '%') continue;
        have_header = true;
        break;
    }
    if (!have_header) {
        *num_nodes = *num_edges = 0;
        return IRR_OK;
    }
    long long n = 0, m = 0;
    if (sscanf(line.c_str(), "%lld %lld", &n, &m) != 2 || n < 0 || m < 0 || n > 0x7fffffffLL)
        return IRR_ERR_ARG;
    int64_t k = 0;
    for (long long i = 0; i < n; i++) {
        if (!std::getline(in, line)) line.clear();
        const char* p = line.c_str();
        for (;;) {
            char* end = nullptr;
            errno = 0;
            const long long v = strtoll(p, &end, 10);
            if (end == p || v <= 0) break;
            p = end;
            if (v - 1 >= i) {  // neighbour j >= i, counted once
                if (v > n) return IRR_ERR_INDEX;
                if (edges && k < cap) {
                    edges[2 * k] = (int32_t)(one_based ? i + 1 : i);
                    edges[2 * k + 1] = (int32_t)(one_based ? v : v - 1);
                }
                k++;
            }
        }
    }
    *num_nodes = n;
    *num_edges = k;
    return k == m ? IRR_OK : IRR_ERR_STATE;
}

int irr_read_coords(const char* path, int64_t num_nodes, double* xyz)
{
    if (!path || num_nodes < 0 || (num_nodes > 0 && !xyz)) return IRR_ERR_ARG;
    FILE* f = fopen(path, "r");
    if (!f) return IRR_ERR_ARG;
    int64_t i = 0;
    double a, b, c;
    while (fscanf(f, "%lf %lf %lf", &a, &b, &c) == 3) {
        if (i < num_nodes) {
            xyz[3 * i] = a;
            xyz[3 * i + 1] = b;
            xyz[3 * i + 2] = c;
        }
        i++;
    }
    fclose(f);
    return i == num_nodes ? IRR_OK : IRR_ERR_STATE;
}

int irr_write_graph(const char* path, int64_t num_nodes, const int32_t* edges, int64_t num_edges)
{
    if (!path || num_nodes < 0 || num_edges < 0 || (num_edges > 0 && !edges)) return IRR_ERR_ARG;
    std::vector<std::vector<int32_t>> adj((size_t)num_nodes);
    int64_t kept = 0;
    for (int64_t t = 0; t < num_edges; t++) {
        const int32_t i = edges[2 * t], j = edges[2 * t + 1];
        if (i < 0 || j < 0 || i >= num_nodes || j >= num_nodes) return IRR_ERR_INDEX;
        adj[(size_t)i].push_back(j);
        if (j != i) adj[(size_t)j].push_back(i);
        kept++;
    }
    FILE* f = fopen(path, "w");
    if (!f) return IRR_ERR_ARG;
    fprintf(f, "%lld %lld\n", (long long)num_nodes, (long long)kept);
    for (int64_t i = 0; i < num_nodes; i++) {
        const std::vector<int32_t>& a = adj[(size_t)i];
        for (size_t k = 0; k < a.size(); k++) fprintf(f, k ? " %d" : "%d", a[k] + 1);
        fputc('\n', f);
    }
    const int bad = ferror(f);
    fclose(f);
    return bad ? IRR_ERR_ARG : IRR_OK;
}

int irr_write_coords(const char* path, int64_t num_nodes, const double* xyz)
{
    if (!path || num_nodes < 0 || (num_nodes > 0 && !xyz)) return IRR_ERR_ARG;
    FILE* f = fopen(path, "w");
    if (!f) return IRR_ERR_ARG;
    for (int64_t i = 0; i < num_nodes; i++)
        fprintf(f, "%.17g %.17g %.17g\n", xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    const int bad = ferror(f);
    fclose(f);
    return bad ? IRR_ERR_ARG : IRR_OK;
}

}  // extern "C"
