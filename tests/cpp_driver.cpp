// cpp_driver.cpp -- test driver for the C++ WFAligner classes
// (include/bindings/cpp/WFAligner.hpp), compiled by the tests.
//
// Usage: cpp_driver <metric> <form> [batch]
//   metric: affine | affine2p | edit | indel | linear
//   form:   e2e | ext | ef:<pattern_begin>,<pattern_end>,<text_begin>,<text_end>
// Reads "pattern<TAB>text" lines from stdin and prints, per pair,
// "status<TAB>score<TAB>operations<TAB>SAM-CIGAR" (per-pair calls), or with
// "batch" one alignBatch() call and "status<TAB>score<TAB>operations".
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "bindings/cpp/WFAligner.hpp"

namespace {
// The protected constructor keeps WFAligner abstract; owning the concrete
// classes through a small holder keeps the driver generic.
std::unique_ptr<wfa::WFAligner, void (*)(wfa::WFAligner*)> make(const std::string& metric) {
  using A = wfa::WFAligner;
  if (metric == "affine2p")
    return {new wfa::WFAlignerGapAffine2Pieces(0, 4, 6, 2, 24, 1, A::Alignment),
            [](A* a) { delete static_cast<wfa::WFAlignerGapAffine2Pieces*>(a); }};
  if (metric == "edit")
    return {new wfa::WFAlignerEdit(A::Alignment),
            [](A* a) { delete static_cast<wfa::WFAlignerEdit*>(a); }};
  if (metric == "indel")
    return {new wfa::WFAlignerIndel(A::Alignment),
            [](A* a) { delete static_cast<wfa::WFAlignerIndel*>(a); }};
  if (metric == "linear")
    return {new wfa::WFAlignerGapLinear(0, 4, 2, A::Alignment),
            [](A* a) { delete static_cast<wfa::WFAlignerGapLinear*>(a); }};
  return {new wfa::WFAlignerGapAffine(0, 4, 6, 2, A::Alignment),
          [](A* a) { delete static_cast<wfa::WFAlignerGapAffine*>(a); }};
}
}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const std::string metric = argv[1], form = argv[2];
  const bool batch = argc > 3 && std::string(argv[3]) == "batch";
  auto al = make(metric);
  al->setHeuristicNone();
  std::vector<std::string> P, T;
  std::string line;
  while (std::getline(std::cin, line)) {
    const size_t tab = line.find('\t');
    if (tab == std::string::npos) continue;
    P.push_back(line.substr(0, tab));
    T.push_back(line.substr(tab + 1));
  }
  if (batch) {
    // the form of the batch is the aligner's current one (end-to-end here)
    std::vector<int> st, sc;
    std::vector<std::string> cig;
    const int rc = al->alignBatch(P, T, st, sc, &cig);
    if (rc != 0) return 3;
    for (size_t i = 0; i < P.size(); ++i)
      std::cout << st[i] << '\t' << sc[i] << '\t' << cig[i] << '\n';
    return 0;
  }
  for (size_t i = 0; i < P.size(); ++i) {
    wfa::WFAligner::AlignmentStatus st;
    if (form == "ext") {
      st = al->alignExtension(P[i], T[i]);
    } else if (form.rfind("ef:", 0) == 0) {
      int pb, pe, tb, te;
      if (std::sscanf(form.c_str() + 3, "%d,%d,%d,%d", &pb, &pe, &tb, &te) != 4) return 2;
      st = al->alignEndsFree(P[i], pb, pe, T[i], tb, te);
    } else {
      st = al->alignEnd2End(P[i], T[i]);
    }
    std::cout << (int)st << '\t' << al->getAlignmentScore() << '\t' << al->getAlignment() << '\t'
              << al->getCIGAR(true) << '\n';
  }
  return 0;
}
