// ptgraph: drop-in command line for the reference's `ptgraph` executable
// (main.cu:4-22, ArgumentParser.cu:15-48). It calls only the C ABI in ascetic.h.
//
// Reference flags, parsed the same way (flag/value pairs from argv[1], unknown
// flags ignored, --type defaults to bfs, --source to 0):
//   --input FILE  --type bfs|sssp|cc|pr  --source N  --adviseK K  --method M (ignored)
// Added flags:
//   --budget-frac F | --budget-bytes B | --budget-edges N   static region size
//   --format auto|bcsr|bwcsr|bcsc|bcsr32
//   --pr-mode ref|std  --precision f64|f32  --max-iter N
//   --output FILE     write the result array (u32 or f64/f32, V entries)
//   --json 1          print one JSON line of run statistics
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "ascetic.h"

static void die(asc_status s, const char *what) {
    char msg[1024];
    asc_last_error(msg, sizeof(msg));
    fprintf(stderr, "ptgraph: %s failed: %s: %s\n", what, asc_status_string(s), msg);
    exit(2);
}

int main(int argc, char **argv) {
    std::string input, algo = "bfs", output, fmt_s = "auto", pr_mode = "ref", precision = "f64";
    long long source = 0;
    double advise = 0, frac = -1, bytes = -1, edges = -1;
    int json = 0, max_iter = 0;
    for (int i = 1; i < argc - 1; i += 2) {
        const char *k = argv[i], *v = argv[i + 1];
        if (!strcmp(k, "--input")) input = v;
        else if (!strcmp(k, "--type")) algo = v;
        else if (!strcmp(k, "--source")) source = atoll(v);
        else if (!strcmp(k, "--adviseK")) advise = atof(v);
        else if (!strcmp(k, "--budget-frac")) frac = atof(v);
        else if (!strcmp(k, "--budget-bytes")) bytes = atof(v);
        else if (!strcmp(k, "--budget-edges")) edges = atof(v);
        else if (!strcmp(k, "--format")) fmt_s = v;
        else if (!strcmp(k, "--pr-mode")) pr_mode = v;
        else if (!strcmp(k, "--precision")) precision = v;
        else if (!strcmp(k, "--max-iter")) max_iter = atoi(v);
        else if (!strcmp(k, "--output")) output = v;
        else if (!strcmp(k, "--json")) json = atoi(v);
        // --method is parsed but unused by the reference; ignored here too
    }
    if (input.empty()) {
        fprintf(stderr,
                "usage: ptgraph --input FILE [--type bfs|sssp|cc|pr] [--source N] [--adviseK K]\n"
                "               [--budget-frac F|--budget-bytes B|--budget-edges N] [--format F]\n"
                "               [--pr-mode ref|std] [--precision f64|f32] [--output FILE] [--json 1]\n");
        return 1;
    }
    asc_algo a;
    if (algo == "bfs") a = ASC_BFS;
    else if (algo == "sssp") a = ASC_SSSP;
    else if (algo == "cc") a = ASC_CC;
    else if (algo == "pr") a = ASC_PR;
    else {
        fprintf(stderr, "ptgraph: unknown --type %s\n", algo.c_str());
        return 1;
    }
    asc_format fmt = ASC_FMT_AUTO;
    if (fmt_s == "bcsr") fmt = ASC_FMT_BCSR;
    else if (fmt_s == "bwcsr") fmt = ASC_FMT_BWCSR;
    else if (fmt_s == "bcsc") fmt = ASC_FMT_BCSC;
    else if (fmt_s == "bcsr32") fmt = ASC_FMT_BCSR32;
    asc_budget b;
    asc_budget_default(&b);
    if (frac >= 0) {
        b.mode = ASC_BUDGET_FRAC;
        b.value = frac;
    } else if (bytes >= 0) {
        b.mode = ASC_BUDGET_BYTES;
        b.value = bytes;
    } else if (edges >= 0) {
        b.mode = ASC_BUDGET_EDGES;
        b.value = edges;
    } else {
        b.mode = ASC_BUDGET_ADVISE_K;
        b.value = advise;
    }
    asc_graph *g = nullptr;
    asc_status s = asc_graph_open(input.c_str(), fmt, &b, &g);
    if (s != ASC_OK) die(s, "open");
    asc_graph_info info;
    asc_graph_info_get(g, &info);
    asc_params p;
    asc_params_default(&p);
    p.pr_mode = pr_mode == "std" ? ASC_PR_STD : ASC_PR_REF;
    p.precision = precision == "f32" ? ASC_F32 : ASC_F64;
    p.max_iterations = max_iter;
    size_t elem = (a == ASC_PR) ? (p.precision == ASC_F32 ? 4 : 8) : 4;
    void *out = malloc(elem * info.vertices);
    if (!out) {
        fprintf(stderr, "ptgraph: out of host memory\n");
        return 2;
    }
    asc_stats st;
    s = asc_run(g, a, (uint32_t)source, &p, out, &st);
    if (s != ASC_OK) die(s, "run");
    printf("vertex num: %llu edge num: %llu\n", (unsigned long long)info.vertices,
           (unsigned long long)info.edges);
    printf("static edges: %llu of %llu, static vertices: %llu\n", (unsigned long long)info.static_edges,
           (unsigned long long)info.edges, (unsigned long long)info.static_vertices);
    printf("iterations: %d\n", st.iterations);
    printf("totalProcess time is %.3f ms\n", st.ms_total);
    printf("move overload size : %llu\n", (unsigned long long)st.ondemand_bytes);
    if (json)
        printf("{\"algo\": \"%s\", \"V\": %llu, \"E\": %llu, \"static_edges\": %llu, \"iterations\": %d, "
               "\"ms\": %.4f, \"edges_processed\": %llu, \"ondemand_bytes\": %llu, \"reached_edges\": %llu, "
               "\"gteps\": %.4f}\n",
               algo.c_str(), (unsigned long long)info.vertices, (unsigned long long)info.edges,
               (unsigned long long)info.static_edges, st.iterations, st.ms_total,
               (unsigned long long)st.edges_processed, (unsigned long long)st.ondemand_bytes,
               (unsigned long long)st.reached_edges, st.ms_total > 0 ? st.reached_edges / st.ms_total / 1e6 : 0.0);
    if (!output.empty()) {
        FILE *f = fopen(output.c_str(), "wb");
        if (!f || fwrite(out, elem, info.vertices, f) != info.vertices) {
            fprintf(stderr, "ptgraph: cannot write %s\n", output.c_str());
            return 2;
        }
        fclose(f);
    }
    free(out);
    asc_graph_close(g);
    return 0;
}
