// Process-level drop-in for the reference's main.x (main.cu:34-95): reads the
// input deck from standard input, the TROVE checkpoints from the working
// directory (or the directory given as the first argument), runs the job on
// one GPU and prints the line list in the reference's format
// (cuda_host.cu:1444-1473) after its header line.
//
//   gi_main [dir] [--split] [--all-j] [--device N] < job.inp > lines.out
//
// --split computes the contractions in split precision (error <= 1e-10 on S);
// --all-j loads every J between the deck's two J values instead of only the two.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

#include "gi.h"

static int die(gi_ctx* c, gi_status s, const char* what) {
  std::fprintf(stderr, "gi_main: %s: %s (%s)\n", what, gi_status_string(s),
               c ? gi_last_error(c) : "");
  if (c) gi_destroy(c);
  return 1;
}

int main(int argc, char** argv) {
  std::string dir = ".";
  bool split = false, all_j = false;
  int device = 0;
  for (int i = 1; i < argc; i++) {
    if (!std::strcmp(argv[i], "--split")) split = true;
    else if (!std::strcmp(argv[i], "--all-j")) all_j = true;
    else if (!std::strcmp(argv[i], "--device") && i + 1 < argc) device = std::atoi(argv[++i]);
    else dir = argv[i];
  }
  const std::string deck_text((std::istreambuf_iterator<char>(std::cin)),
                              std::istreambuf_iterator<char>());
  gi_deck deck;
  char err[512] = {0};
  gi_status st = gi_deck_parse(deck_text.c_str(), &deck, err, sizeof(err));
  if (st != GI_OK) {
    std::fprintf(stderr, "gi_main: deck: %s\n", err);
    return 1;
  }
  deck.params.precision = split ? GI_PREC_SPLIT : GI_PREC_FP64;
  gi_ctx* c = nullptr;
  if ((st = gi_create(&c, device, 0)) != GI_OK) return die(nullptr, st, "gi_create");
  if ((st = gi_load_trove(c, dir.c_str(), &deck, all_j ? GI_TROVE_ALL_J : 0)) != GI_OK)
    return die(c, st, "gi_load_trove");
  int64_t n = 0;
  if ((st = gi_run(c, 0, &n)) != GI_OK) return die(c, st, "gi_run");
  if ((st = gi_sort_lines(c)) != GI_OK) return die(c, st, "gi_sort_lines");
  std::printf("Linestrength S(f<-i) [Debye**2], Transition moments [Debye],Einstein "
              "coefficient A(if) [1/s],and Intensities [cm/mol]\n\n\n");
  const int64_t chunk = 1 << 16;
  std::vector<char> buf;
  for (int64_t off = 0; off < n; off += chunk) {
    const int64_t cnt = n - off < chunk ? n - off : chunk;
    size_t used = 0;
    if ((st = gi_format_lines(c, off, cnt, nullptr, 0, &used)) != GI_OK)
      return die(c, st, "gi_format_lines");
    buf.resize(used + 1);
    if ((st = gi_format_lines(c, off, cnt, buf.data(), buf.size(), &used)) != GI_OK)
      return die(c, st, "gi_format_lines");
    std::fwrite(buf.data(), 1, used, stdout);
  }
  gi_destroy(c);
  return 0;
}
