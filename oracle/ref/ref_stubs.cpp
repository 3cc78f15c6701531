// ref_stubs.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Definitions of the few symbols that the IFEM sources compiled for the
// reference build (oracle/ref/build_ref.py) reference but that live in IFEM
// translation units which cannot be built here (they need tinyxml2, CBLAS or
// GoTools).  None of them is on the assembly path that the harness drives,
// except utl::getDigits, which ASMbase::fix uses to split a DOF code such as
// 123 into its digits and which is therefore implemented for real.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <map>
#include <set>
#include <vector>

#include "ASM2D.h"
#include "ASM3D.h"
#include "IFEM.h"
#include "LinAlgInit.h"
#include "LogStream.h"
#include "Utilities.h"

namespace {
[[noreturn]] void unavailable(const char* what)
{
  std::fprintf(stderr, "reference build: %s is not part of this build\n", what);
  std::abort();
}
}  // namespace

utl::LogStream IFEM::cout(std::cout);
void IFEM::Close() {}

int LinAlgInit::refs = 0;
LinAlgInit* LinAlgInit::instance = nullptr;
LinAlgInit::~LinAlgInit() {}

ASMbase* ASM2D::clone(const CharVec&) const { unavailable("ASM2D::clone"); }
ASMbase* ASM3D::clone(const CharVec&) const { unavailable("ASM3D::clone"); }

// The decimal digits of value, e.g. 123 -> {1, 2, 3} (semantics of
// src/Utility/Utilities.h:214).
std::set<int> utl::getDigits(int value)
{
  std::set<int> digits;
  for (; value > 0; value /= 10) digits.insert(value % 10);
  return digits;
}

bool utl::parseIntegers(std::vector<int>&, const char*) { unavailable("utl::parseIntegers"); }
bool utl::renumber(int&, int&, IntMap&) { unavailable("utl::renumber"); }
bool utl::renumber(int&, const IntMap&, bool) { unavailable("utl::renumber"); }
int utl::findKey(const IntMap&, int) { unavailable("utl::findKey"); }
int utl::findIndex(const std::vector<int>&, int) { unavailable("utl::findIndex"); }
