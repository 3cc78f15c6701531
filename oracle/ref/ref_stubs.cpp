// ref_stubs.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Definitions of the few symbols that the IFEM sources compiled for the
// reference build (oracle/ref/build_ref.py) reference but that live in IFEM
// translation units which cannot be built here (they need tinyxml2, CBLAS or
// GoTools).  Three of them are on the path the harness drives and are
// implemented from their documented behaviour (src/Utility/Utilities.h):
// utl::getDigits (ASMbase::fix splits a DOF code such as 123 into digits)
// and the two utl::renumber overloads (node merging and renumbering of
// connected patches, ASMbase::mergeNodes / renumberNodes).
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
// A value not seen before becomes ++runner; returns whether num changed.
bool utl::renumber(int& num, int& runner, IntMap& old2new)
{
  auto it = old2new.find(num);
  if (it == old2new.end()) it = old2new.emplace(num, ++runner).first;
  const bool changed = num != it->second;
  num = it->second;
  return changed;
}

// num mapped through old2new; returns whether num was in the mapping.
bool utl::renumber(int& num, const IntMap& old2new, bool msg)
{
  auto it = old2new.find(num);
  if (it == old2new.end()) {
    if (msg) std::fprintf(stderr, "utl::renumber: %d not in the mapping\n", num);
    return false;
  }
  num = it->second;
  return true;
}
int utl::findKey(const IntMap&, int) { unavailable("utl::findKey"); }
int utl::findIndex(const std::vector<int>&, int) { unavailable("utl::findIndex"); }
