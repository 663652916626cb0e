/*
 * ref_spm.cc : the reference's hit-merge functors run through thrust on the host (TEST INFRASTRUCTURE ONLY).
 *
 * Built by `make -C oracle ref-spm` into oracle/_ref/ref_spm (git-ignored) with the host compiler on thrust's CPP
 * backend, from the reference's unmodified sysrap/sphoton.h: its sphoton::select_pred, sphoton::key_functor and
 * sphoton::reduce_op (sphoton.h:277-304) drive the step sequence of SPM::merge_partial_select
 * (sysrap/SPM.cu:135-250):
 *   select (count_if + copy_if with select_pred), keys by key_functor{time_window}, sort_by_key of the selected
 *   photons by key, reduce_by_key with equal_to<uint64_t> and reduce_op; time_window 0 returns the selection.
 * SPM.cu itself runs only on the CUDA backend (thrust::cuda::par_nosync, stream-ordered allocations), so the steps
 * are restated here around the same functors.  The CUDA backend sorts 64-bit keys with a stable radix sort, so
 * the restatement sorts stably.
 *
 * Usage: ref_spm <photons.bin> <select_flagmask> <time_window_ns> <merged.bin>
 * Reads and writes raw arrays of 64-byte sphoton records.
 */
#include <cstdint>
#include <cstdio>
#include <vector>

#include <vector_types.h>
#include <vector_functions.h>
#include "scuda.h"
#include "squad.h"
#include "sphoton.h"

#include <thrust/copy.h>
#include <thrust/count.h>
#include <thrust/functional.h>
#include <thrust/host_vector.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/reduce.h>
#include <thrust/sort.h>

int main(int argc, char** argv)
{
    if (argc < 5) { std::fprintf(stderr, "usage: ref_spm photons.bin select_flagmask time_window out.bin\n"); return 2; }
    const unsigned mask = (unsigned)std::strtoul(argv[2], nullptr, 0);
    const float tw = std::strtof(argv[3], nullptr);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    std::fseek(f, 0, SEEK_END);
    const long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    thrust::host_vector<sphoton> in((size_t)bytes / sizeof(sphoton));
    if (std::fread(in.data(), sizeof(sphoton), in.size(), f) != in.size()) return 4;
    std::fclose(f);

    sphoton::select_pred selector{mask};
    const size_t num_selected = (size_t)thrust::count_if(in.begin(), in.end(), selector);
    thrust::host_vector<sphoton> sel(num_selected);
    thrust::copy_if(in.begin(), in.end(), sel.begin(), selector);
    thrust::host_vector<sphoton> out;
    if (tw == 0.f || num_selected == 0) {
        out = sel;
    } else {
        thrust::host_vector<uint64_t> keys(num_selected);
        auto k = thrust::make_transform_iterator(sel.begin(), sphoton::key_functor{tw});
        thrust::copy(k, k + num_selected, keys.begin());
        thrust::stable_sort_by_key(keys.begin(), keys.end(), sel.begin());
        thrust::host_vector<uint64_t> out_key(num_selected);
        out.resize(num_selected);
        auto ends = thrust::reduce_by_key(keys.begin(), keys.end(), sel.begin(), out_key.begin(), out.begin(),
                                          thrust::equal_to<uint64_t>{}, sphoton::reduce_op{});
        out.resize((size_t)(ends.first - out_key.begin()));
    }
    FILE* g = std::fopen(argv[4], "wb");
    if (!g) return 5;
    if (!out.empty() && std::fwrite(out.data(), sizeof(sphoton), out.size(), g) != out.size()) return 6;
    std::fclose(g);
    std::printf("%zu %zu %zu\n", in.size(), num_selected, out.size());
    return 0;
}
