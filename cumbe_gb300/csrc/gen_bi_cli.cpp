// `gen_bi <edges> <out.bi> [skip_words] [skip_words_per_edge]` - drop-in for
// the reference's KONECT converter (data/gen_bi.cpp): same arguments, same
// prompts when the two counts are not given, same `.bi` graph out (row
// lists sorted; the reference writes them in hash-set order).  Errors go to
// stderr with exit status 1.
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "mbe.h"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cout << "Wrong Dataset :(\n";
        return 0;
    }
    long skip = 0, skip_edge = 0;
    std::cout << "Number of passed words: ";
    if (argc > 3)
        std::cout << (skip = std::atol(argv[3])) << "\n";
    else
        std::cin >> skip;
    std::cout << "Number of passed words per edge: ";
    if (argc > 4)
        std::cout << (skip_edge = std::atol(argv[4])) << "\n";
    else
        std::cin >> skip_edge;
    if (skip < 0 || skip_edge < 0) {
        std::fprintf(stderr, "gen_bi: negative counts\n");
        return 1;
    }
    mbe_graph* g = nullptr;
    mbe_status st = mbe_graph_load_konect(argv[1], (uint32_t)skip, (uint32_t)skip_edge, &g);
    if (st != MBE_OK) {
        std::fprintf(stderr, "gen_bi: %s\n", mbe_last_error());
        return 1;
    }
    std::cout << "Loading... Done\nWriting..." << std::flush;
    st = mbe_graph_write_bi(g, argv[2]);
    mbe_graph_free(g);
    if (st != MBE_OK) {
        std::fprintf(stderr, "gen_bi: %s\n", mbe_last_error());
        return 1;
    }
    std::cout << " Done\n";
    return 0;
}
