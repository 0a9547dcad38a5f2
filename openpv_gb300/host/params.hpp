// params.hpp -- a reader of OpenPV params files (the grammar of io/parser/params.l and
// params.y): top-level directives `name = number;`, parameter groups
// `Keyword "name" = { ... };` holding numbers, strings, file names and number arrays,
// `#include "group";` (copies an earlier group's parameters; first entry of a group only),
// `@name = value;` overrides of included parameters, `//` comments, `infinity` (= FLT_MAX),
// `true` / `false`, `NULL`.  ParameterSweep groups are read and kept but not expanded.
#pragma once

#include <string>
#include <utility>
#include <vector>

namespace pvhost {

struct ParamValue {
   enum Kind { Number, String, Array } kind = Number;
   double number = 0.0;
   std::string str;
   bool null = false;  // NULL string
   std::vector<double> array;
};

struct ParamGroup {
   std::string keyword, name;
   std::vector<std::pair<std::string, ParamValue>> params;  // in file order
   bool sweep = false;

   const ParamValue *find(const std::string &key) const;
   bool has(const std::string &key) const { return find(key) != nullptr; }
   double number(const std::string &key, double dflt) const;
   bool flag(const std::string &key, bool dflt) const { return number(key, dflt ? 1.0 : 0.0) != 0.0; }
   std::string string(const std::string &key, const std::string &dflt) const;
};

struct Params {
   std::vector<std::pair<std::string, double>> directives;
   std::vector<ParamGroup> groups;
   const ParamGroup *group(const std::string &name) const;
};

// Parses `text`; on failure returns false with a message naming the line.
bool parse_params(const std::string &text, Params &out, std::string &error);

// A canonical one-line-per-parameter rendering (for tests).
std::string dump_params(const Params &p);

}  // namespace pvhost
