// params.cpp -- tokenizer and recursive-descent reader for the OpenPV params grammar (see
// params.hpp).  Token classes follow io/parser/params.l: numbers with optional sign, fraction
// and exponent; `infinity` / `+infinity` / `-infinity` as +-FLT_MAX; `true` / `false` as 1 / 0;
// identifiers; `@identifier` overrides; double-quoted strings; the punctuation { } [ ] = , ; :.
#include "params.hpp"

#include <cctype>
#include <cstring>
#include <cfloat>
#include <cstdlib>
#include <sstream>

namespace pvhost {

const ParamValue *ParamGroup::find(const std::string &key) const {
   for (const auto &kv : params)
      if (kv.first == key) return &kv.second;
   return nullptr;
}

double ParamGroup::number(const std::string &key, double dflt) const {
   const ParamValue *v = find(key);
   return v && v->kind == ParamValue::Number ? v->number : dflt;
}

std::string ParamGroup::string(const std::string &key, const std::string &dflt) const {
   const ParamValue *v = find(key);
   return v && v->kind == ParamValue::String && !v->null ? v->str : dflt;
}

const ParamGroup *Params::group(const std::string &name) const {
   for (const auto &g : groups)
      if (g.name == name && !g.sweep) return &g;
   return nullptr;
}

namespace {

enum Tok { T_END, T_NUMBER, T_ID, T_OVERWRITE, T_STRING, T_NULL, T_INCLUDE, T_SWEEP, T_PUNCT, T_BAD };

struct Token {
   Tok kind = T_END;
   std::string text;
   double number = 0.0;
   int line = 1;
};

class Lexer {
 public:
   explicit Lexer(const std::string &s) : s_(s) {}

   Token next() {
      skip();
      Token t;
      t.line = line_;
      if (i_ >= s_.size()) return t;
      const char c = s_[i_];
      if (c == '#') {
         if (s_.compare(i_, 8, "#include") == 0) {
            i_ += 8;
            t.kind = T_INCLUDE;
            return t;
         }
         return bad(t);
      }
      if (c == '@') {
         size_t j = i_ + 1;
         if (j < s_.size() && std::isalpha((unsigned char)s_[j])) {
            while (j < s_.size() && (std::isalnum((unsigned char)s_[j]) || s_[j] == '_')) j++;
            t.kind = T_OVERWRITE;
            t.text = s_.substr(i_ + 1, j - i_ - 1);
            i_ = j;
            return t;
         }
         return bad(t);
      }
      if (c == '"') {
         size_t j = s_.find('"', i_ + 1);
         if (j == std::string::npos) return bad(t);
         t.kind = T_STRING;
         t.text = s_.substr(i_ + 1, j - i_ - 1);
         i_ = j + 1;
         return t;
      }
      if (std::strchr("{}[]=,;:", c)) {
         t.kind = T_PUNCT;
         t.text = std::string(1, c);
         i_++;
         return t;
      }
      // signed infinity
      for (const char *w : {"+infinity", "-infinity", "infinity"}) {
         const size_t n = std::strlen(w);
         if (s_.compare(i_, n, w) == 0 && !idchar(i_ + n)) {
            t.kind = T_NUMBER;
            t.number = w[0] == '-' ? -FLT_MAX : FLT_MAX;
            i_ += n;
            return t;
         }
      }
      if (std::isdigit((unsigned char)c) || c == '.' || ((c == '+' || c == '-') && i_ + 1 < s_.size() &&
                                                         (std::isdigit((unsigned char)s_[i_ + 1]) || s_[i_ + 1] == '.'))) {
         const char *start = s_.c_str() + i_;
         char *end = nullptr;
         t.number = std::strtod(start, &end);
         if (end == start) return bad(t);
         t.kind = T_NUMBER;
         i_ += (size_t)(end - start);
         return t;
      }
      if (std::isalpha((unsigned char)c)) {
         size_t j = i_;
         while (j < s_.size() && (std::isalnum((unsigned char)s_[j]) || s_[j] == '_')) j++;
         t.text = s_.substr(i_, j - i_);
         i_ = j;
         if (t.text == "true" || t.text == "false") {
            t.kind = T_NUMBER;
            t.number = t.text == "true" ? 1.0 : 0.0;
         } else if (t.text == "NULL") {
            t.kind = T_NULL;
         } else if (t.text == "ParameterSweep") {
            t.kind = T_SWEEP;
         } else {
            t.kind = T_ID;
         }
         return t;
      }
      return bad(t);
   }

 private:
   bool idchar(size_t j) const { return j < s_.size() && (std::isalnum((unsigned char)s_[j]) || s_[j] == '_'); }
   Token bad(Token t) {
      t.kind = T_BAD;
      t.text = std::string(1, s_[i_]);
      i_++;
      return t;
   }
   void skip() {
      while (i_ < s_.size()) {
         const char c = s_[i_];
         if (c == '\n') {
            line_++;
            i_++;
         } else if (std::isspace((unsigned char)c)) {
            i_++;
         } else if (c == '/' && i_ + 1 < s_.size() && s_[i_ + 1] == '/') {
            while (i_ < s_.size() && s_[i_] != '\n') i_++;
         } else {
            break;
         }
      }
   }
   const std::string &s_;
   size_t i_ = 0;
   int line_ = 1;
};

class Parser {
 public:
   Parser(const std::string &text, Params &out) : lex_(text), out_(out) { advance(); }

   bool parse(std::string &err) {
      while (cur_.kind != T_END) {
         if (cur_.kind == T_SWEEP) {
            if (!sweep()) return fail(err);
         } else if (cur_.kind == T_ID) {
            Token id = cur_;
            advance();
            if (cur_.kind == T_STRING) {
               if (!group(id)) return fail(err);
            } else if (punct("=")) {
               advance();
               if (cur_.kind != T_NUMBER) return expected("a number", err);
               out_.directives.push_back({id.text, cur_.number});
               advance();
               if (!take(";")) return expected("';'", err);
            } else {
               return expected("a group name or '='", err);
            }
         } else {
            return expected("a parameter group", err);
         }
      }
      return true;
   }

 private:
   void advance() { cur_ = lex_.next(); }
   bool punct(const char *p) const { return cur_.kind == T_PUNCT && cur_.text == p; }
   bool take(const char *p) {
      if (!punct(p)) return false;
      advance();
      return true;
   }
   bool expected(const char *what, std::string &err) {
      std::ostringstream o;
      o << "params line " << cur_.line << ": expected " << what << " near '" << cur_.text << "'";
      err = o.str();
      return false;
   }
   bool fail(std::string &err) {
      if (err.empty()) {
         std::ostringstream o;
         o << "params line " << cur_.line << ": " << (msg_.empty() ? "syntax error" : msg_) << " near '" << cur_.text
           << "'";
         err = o.str();
      }
      return false;
   }

   bool value(ParamValue &v) {
      if (cur_.kind == T_NUMBER) {
         v.kind = ParamValue::Number;
         v.number = cur_.number;
         advance();
         return true;
      }
      if (cur_.kind == T_STRING) {
         v.kind = ParamValue::String;
         v.str = cur_.text;
         advance();
         return true;
      }
      if (cur_.kind == T_NULL) {
         v.kind = ParamValue::String;
         v.null = true;
         advance();
         return true;
      }
      if (take("[")) {
         v.kind = ParamValue::Array;
         if (take("]")) return true;
         for (;;) {
            if (cur_.kind != T_NUMBER) return false;
            v.array.push_back(cur_.number);
            advance();
            if (take("]")) return true;
            if (!take(",")) return false;
         }
      }
      return false;
   }

   bool group(const Token &keyword) {
      ParamGroup g;
      g.keyword = keyword.text;
      g.name = cur_.text;
      advance();
      if (!take("=") || !take("{")) return false;
      bool first = true;
      while (!punct("}")) {
         if (cur_.kind == T_INCLUDE) {
            advance();
            if (cur_.kind != T_STRING) return false;
            if (!first) {
               msg_ = "#include must be the first entry of a group";
               return false;
            }
            const ParamGroup *src = out_.group(cur_.text);
            if (!src) {
               msg_ = "#include of an unknown group";
               return false;
            }
            g.params = src->params;
            advance();
            if (!take(";")) return false;
         } else if (cur_.kind == T_ID || cur_.kind == T_OVERWRITE) {
            const bool over = cur_.kind == T_OVERWRITE;
            const std::string key = cur_.text;
            advance();
            if (!take("=")) return false;
            ParamValue v;
            if (!value(v) || !take(";")) return false;
            bool found = false;
            for (auto &kv : g.params)
               if (kv.first == key) {
                  if (!over) {
                     msg_ = "parameter defined twice in a group";
                     return false;
                  }
                  kv.second = v;
                  found = true;
               }
            if (over && !found) {
               msg_ = "@ override of a parameter the group does not have";
               return false;
            }
            if (!found) g.params.push_back({key, v});
         } else {
            return false;
         }
         first = false;
      }
      advance();  // '}'
      if (!take(";")) return false;
      if (out_.group(g.name)) {
         msg_ = "two groups with the same name";
         return false;
      }
      out_.groups.push_back(std::move(g));
      return true;
   }

   // ParameterSweep "group":param = { v; v; ... };  -- kept, not expanded
   bool sweep() {
      advance();
      if (cur_.kind != T_STRING) return false;
      ParamGroup g;
      g.keyword = "ParameterSweep";
      g.name = cur_.text;
      g.sweep = true;
      advance();
      if (!take(":") || cur_.kind != T_ID) return false;
      const std::string key = cur_.text;
      advance();
      if (!take("=") || !take("{")) return false;
      ParamValue arr;
      arr.kind = ParamValue::Array;
      while (!punct("}")) {
         ParamValue v;
         if (!value(v) || !take(";")) return false;
         if (v.kind == ParamValue::Number) arr.array.push_back(v.number);
      }
      advance();
      if (!take(";")) return false;
      g.params.push_back({key, arr});
      out_.groups.push_back(std::move(g));
      return true;
   }

   Lexer lex_;
   Params &out_;
   Token cur_;
   std::string msg_;
};

}  // namespace

bool parse_params(const std::string &text, Params &out, std::string &error) {
   out = Params();
   error.clear();
   Parser p(text, out);
   return p.parse(error);
}

std::string dump_params(const Params &p) {
   std::ostringstream o;
   o.precision(9);
   for (const auto &d : p.directives) o << d.first << " = " << d.second << "\n";
   for (const auto &g : p.groups) {
      o << g.keyword << " \"" << g.name << "\"\n";
      for (const auto &kv : g.params) {
         o << "  " << kv.first << " = ";
         const ParamValue &v = kv.second;
         if (v.kind == ParamValue::Number) o << v.number;
         else if (v.kind == ParamValue::String) o << (v.null ? std::string("NULL") : "\"" + v.str + "\"");
         else {
            o << "[";
            for (size_t i = 0; i < v.array.size(); i++) o << (i ? ", " : "") << v.array[i];
            o << "]";
         }
         o << "\n";
      }
   }
   return o.str();
}

}  // namespace pvhost
