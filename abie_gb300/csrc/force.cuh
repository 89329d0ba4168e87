// All-pairs Newtonian acceleration on the GPU: launchers shared by the C ABI,
// the Radau15 engine and the benchmarks.
#pragma once
#include "common.cuh"

namespace abie {

// Scratch for one standalone force evaluation: the compact list of massive
// sources (position, G m) in body order, their body indices and count.
struct ForceScratch {
    Src *src = nullptr;
    int *src_body = nullptr;
    int *n_src = nullptr;       // device scalar
    double *partial = nullptr;  // per (sink, source chunk) partial sums, 3 doubles each
    unsigned long long *gm_max = nullptr;  // mixed form: largest G m (as ordered bits)
    float *mixed_soa = nullptr;            // mixed form: anchored two-float sources
    size_t mixed_cap = 0;                  // floats
    unsigned int *next = nullptr;          // fp64 form: next sink to hand out
    int *counts = nullptr;      // parallel compaction: massive bodies per chunk
    // symmetric form (every body massive): work items, first item per row,
    // partial sums of the items' sinks and source tiles
    int2 *sym_items = nullptr;
    int *sym_row = nullptr;
    double *sym_apart = nullptr, *sym_bpart = nullptr;
    int sym_n = 0, sym_nt = 0, sym_items_n = 0;
    size_t cap = 0;             // bodies
    size_t partial_cap = 0;     // doubles
};

int force_scratch_reserve(ForceScratch &s, size_t n);
void force_scratch_free(ForceScratch &s);

// Order-preserving compaction of the bodies with m > 0 (src/common.c:60:
// only positive masses act as sources).
int launch_compact_sources(const double *pos, const double *m, int n, double G, Src *src,
                           int *src_body, int *n_src, cudaStream_t st);
// The same list built by many blocks (a count pass and a scatter pass),
// for n above a few thousand bodies; counts holds one int per 2,048 bodies.
int launch_compact_sources_parallel(const double *pos, const double *m, int n, double G, Src *src,
                                    int *src_body, int *n_src, int *counts, cudaStream_t st);

// acc[3j..3j+2] for every sink j in [0, n).  Sinks with m < 0 are skipped
// (their entries are not written), as in src/common.c:49-52.
int launch_force(int mode, const double *pos, const double *m, int n, double G,
                 ForceScratch &s, double *acc, cudaStream_t st);

// Fast FP64 force of the n sinks at pos against a source list already built
// (*n_src_dev records, e.g. the Radau15 engine's published substep), with
// lanes (1, 8 or 32) per sink and sinks handed out from the counter next
// (zeroed here): the same sums, in the same order, as the persistent
// engine's sink loop with that many lanes per body.  With 32 lanes and a
// partial-sum buffer (6 n doubles) each sink's sources split in two chunks
// instead (the standalone force's form from 8,192 sinks).
int launch_force_published(const double *pos, const double *m, int n, const Src *src,
                           const int *n_src_dev, int lanes, double *acc, unsigned int *next,
                           cudaStream_t st, double *partial = nullptr);

// The symmetric form (each pair once for both bodies) on a published source
// list that holds every body in body order (*n_src_dev == n), with the
// symmetric scratch of s; force_sym_applies says whether it is used for a
// system of n bodies and n_src massive ones.
int launch_force_published_sym(const Src *src, int n, const int *n_src_dev, double *acc,
                               ForceScratch &s, cudaStream_t st);
bool force_sym_applies(int n, int n_src);

// Fast FP64 force with caller-provided scratch (src / src_body sized for n
// entries, n_src one int); allocates nothing.  Uses one source chunk.
int launch_force_fp64_scratch(const double *pos, const double *m, int n, double G, Src *src,
                              int *src_body, int *n_src, double *acc, cudaStream_t st);

// Launch shape of the fast FP64 kernel, exposed for the autotuner.
struct ForceShape {
    int lanes_per_sink;   // 1, 8 or 32
    int chunks;           // source chunks per sink (1 = no split)
};
ForceShape force_shape_default(int n_sink, int n_src);  // honours abie_debug_force_shape
ForceShape force_shape_auto(int n_sink, int n_src);     // the automatic choice only
void force_shape_override(int lanes_per_sink, int chunks);  // 0,0 = automatic

// Energy (src/common.c:340-357) of a state on the device, FP64.
int launch_energy(const double *pos, const double *vel, const double *m, int n, double G,
                  double *d_partials, double *h_out, cudaStream_t st);

}  // namespace abie
