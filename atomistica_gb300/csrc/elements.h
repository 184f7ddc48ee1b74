// Chemical element symbols by atomic number (host side): the lookups behind
// the setfl header check (tabulated_alloy_eam.f90:206-213, ElementName) and
// the element filters of the EAM potentials (filter_from_string,
// src/core/filter.f90:55-120, atomic_number).
#pragma once

#include <cstring>
#include <string>

namespace gb {

inline const char *element_name(int Z) {
  static const char *const kNames[] = {
      "X",  "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si",
      "P",  "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu",
      "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru",
      "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr",
      "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",
      "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac",
      "Th", "Pa", "U",  "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm", "Md", "No", "Lr", "Rf",
      "Db", "Sg", "Bh", "Hs", "Mt", "Ds", "Rg", "Cn", "Nh", "Fl", "Mc", "Lv", "Ts", "Og"};
  constexpr int kMaxZ = (int)(sizeof(kNames) / sizeof(kNames[0])) - 1;
  return (Z >= 1 && Z <= kMaxZ) ? kNames[Z] : nullptr;
}

// atomic_number_from_symbol (PeriodicTable.f90:134-157): leading blanks
// dropped, a string of digits is an atomic number, otherwise the symbol is
// matched without regard to case; 0 if unknown.
inline int element_Z(const std::string &sym_in) {
  std::string sym = sym_in;
  sym.erase(0, sym.find_first_not_of(' '));
  sym.erase(sym.find_last_not_of(' ') + 1);
  if (sym.empty()) return 0;
  if (sym.find_first_not_of("0123456789") == std::string::npos) {
    const int Z = sym.size() > 3 ? 0 : std::stoi(sym);
    return element_name(Z) ? Z : 0;
  }
  auto lower = [](std::string x) {
    for (auto &c : x) c = (char)((c >= 'A' && c <= 'Z') ? c - 'A' + 'a' : c);
    return x;
  };
  const std::string l = lower(sym);
  for (int Z = 1; element_name(Z); Z++)
    if (l == lower(element_name(Z))) return Z;
  return 0;
}

}  // namespace gb
