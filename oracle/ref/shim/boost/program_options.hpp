// Minimal stand-in for the subset of boost::program_options that the
// reference's mcmc/options.h and dkvstore/DKVStore.h use, written for the
// oracle's reference build (test infrastructure only).  Behaviour kept:
// long/short names, default values, bool switches, allow_unregistered,
// collect_unrecognized, config files, first store wins, notify() writes the
// bound variables, validate<T> customisation point.
#pragma once
#include <any>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace boost {
using any = std::any;
template <class E>
[[noreturn]] inline void throw_exception(const E& e) {
  throw e;
}
namespace program_options {

class error : public std::logic_error {
 public:
  explicit error(const std::string& w) : std::logic_error(w) {}
};

class validation_error : public error {
 public:
  enum kind_t {
    multiple_values_not_allowed = 30,
    at_least_one_value_required,
    invalid_bool_value,
    invalid_option_value,
    invalid_option
  };
  explicit validation_error(kind_t, const std::string& opt = "", const std::string& = "")
      : error("validation error: " + opt) {}
};

class invalid_option_value : public validation_error {
 public:
  explicit invalid_option_value(const std::string& bad)
      : validation_error(validation_error::invalid_option_value, bad) {}
};

namespace validators {
inline void check_first_occurrence(const boost::any& v) {
  if (v.has_value()) throw validation_error(validation_error::multiple_values_not_allowed);
}
inline const std::string& get_single_string(const std::vector<std::string>& v) {
  if (v.size() != 1) throw validation_error(validation_error::invalid_option_value);
  return v[0];
}
}  // namespace validators

template <class T, class charT>
void validate(boost::any& v, const std::vector<std::basic_string<charT> >& xs, T*, long) {
  validators::check_first_occurrence(v);
  const std::string& s = validators::get_single_string(xs);
  std::istringstream is(s);
  T x;
  if (!(is >> x)) throw invalid_option_value(s);
  v = boost::any(x);
}

template <class charT>
void validate(boost::any& v, const std::vector<std::basic_string<charT> >& xs, std::string*, long) {
  validators::check_first_occurrence(v);
  v = boost::any(validators::get_single_string(xs));
}

class value_semantic {
 public:
  virtual ~value_semantic() {}
  virtual void parse(boost::any& v, const std::vector<std::string>& tokens) const = 0;
  virtual bool apply_default(boost::any& v) const = 0;
  virtual void notify(const boost::any& v) const = 0;
  virtual bool is_switch() const { return false; }
};

template <class T>
class typed_value : public value_semantic {
 public:
  explicit typed_value(T* store) : store_(store) {}
  typed_value* default_value(const T& v) {
    has_default_ = true;
    default_ = v;
    return this;
  }
  typed_value* multitoken() { return this; }
  void parse(boost::any& v, const std::vector<std::string>& tokens) const override {
    if (switch_) {
      v = boost::any(true);
      return;
    }
    validate(v, tokens, (T*)0, 0L);
  }
  bool apply_default(boost::any& v) const override {
    if (!has_default_) return false;
    v = boost::any(default_);
    return true;
  }
  void notify(const boost::any& v) const override {
    if (store_ && v.has_value()) *store_ = std::any_cast<T>(v);
  }
  bool is_switch() const override { return switch_; }
  bool switch_ = false;

 private:
  T* store_;
  bool has_default_ = false;
  T default_{};
};

template <class T>
typed_value<T>* value(T* store) {
  return new typed_value<T>(store);
}

inline typed_value<bool>* bool_switch(bool* store) {
  auto* v = new typed_value<bool>(store);
  v->switch_ = true;
  v->default_value(false);
  return v;
}

struct option_description {
  std::string long_name, short_name, text;
  std::shared_ptr<value_semantic> semantic;
};

class options_description {
 public:
  explicit options_description(const std::string& caption = "") : caption_(caption) {}
  struct easy_init {
    options_description* d;
    easy_init& operator()(const char* name, const value_semantic* s, const char* text = "") {
      auto o = std::make_shared<option_description>();
      std::string n(name);
      auto c = n.find(',');
      o->long_name = n.substr(0, c);
      if (c != std::string::npos) o->short_name = n.substr(c + 1);
      o->text = text;
      o->semantic.reset(const_cast<value_semantic*>(s));
      d->opts_.push_back(o);
      return *this;
    }
  };
  easy_init add_options() { return easy_init{this}; }
  options_description& add(const options_description& other) {
    opts_.insert(opts_.end(), other.opts_.begin(), other.opts_.end());
    return *this;
  }
  const option_description* find(const std::string& key, bool short_name) const {
    for (auto& o : opts_)
      if ((short_name ? o->short_name : o->long_name) == key && !key.empty()) return o.get();
    return nullptr;
  }
  const std::vector<std::shared_ptr<option_description> >& options() const { return opts_; }
  const std::string& caption() const { return caption_; }

 private:
  std::string caption_;
  std::vector<std::shared_ptr<option_description> > opts_;
};

inline std::ostream& operator<<(std::ostream& os, const options_description& d) {
  os << d.caption() << ":\n";
  for (auto& o : d.options())
    os << "  --" << o->long_name << (o->short_name.empty() ? "" : " [-" + o->short_name + "]")
       << "  " << o->text << "\n";
  return os;
}

struct option {
  std::string string_key;
  std::vector<std::string> value;
  std::vector<std::string> original_tokens;
  bool unregistered = false;
};

struct parsed_options {
  std::vector<option> options;
  const options_description* description = nullptr;
};

enum collect_unrecognized_mode { include_positional, exclude_positional };

inline std::vector<std::string> collect_unrecognized(const std::vector<option>& opts,
                                                     collect_unrecognized_mode) {
  std::vector<std::string> r;
  for (auto& o : opts)
    if (o.unregistered) r.insert(r.end(), o.original_tokens.begin(), o.original_tokens.end());
  return r;
}

class command_line_parser {
 public:
  explicit command_line_parser(const std::vector<std::string>& args) : args_(args) {}
  command_line_parser& options(const options_description& d) {
    desc_ = &d;
    return *this;
  }
  command_line_parser& allow_unregistered() {
    allow_ = true;
    return *this;
  }
  parsed_options run() {
    parsed_options p;
    p.description = desc_;
    for (size_t i = 0; i < args_.size(); ++i) {
      const std::string& t = args_[i];
      const option_description* d = nullptr;
      std::string inline_val;
      bool has_inline = false;
      if (t.size() > 2 && t[0] == '-' && t[1] == '-') {
        std::string n = t.substr(2);
        auto eq = n.find('=');
        if (eq != std::string::npos) {
          inline_val = n.substr(eq + 1);
          has_inline = true;
          n = n.substr(0, eq);
        }
        d = desc_->find(n, false);
      } else if (t.size() >= 2 && t[0] == '-') {
        d = desc_->find(t.substr(1, 1), true);
        if (d && t.size() > 2) {
          inline_val = t.substr(2);
          has_inline = true;
        }
      }
      option o;
      o.original_tokens.push_back(t);
      if (!d) {
        if (!allow_) throw error("unrecognised option " + t);
        o.unregistered = true;
        p.options.push_back(o);
        continue;
      }
      o.string_key = d->long_name;
      if (!d->semantic->is_switch()) {
        if (has_inline) {
          o.value.push_back(inline_val);
        } else {
          if (i + 1 >= args_.size()) throw error("missing value for " + t);
          o.value.push_back(args_[++i]);
          o.original_tokens.push_back(args_[i]);
        }
      }
      p.options.push_back(o);
    }
    return p;
  }

 private:
  std::vector<std::string> args_;
  const options_description* desc_ = nullptr;
  bool allow_ = false;
};

struct variable_value {
  boost::any v;
  bool defaulted = false;
  const value_semantic* semantic = nullptr;
};

class variables_map : public std::map<std::string, variable_value> {};

inline void store(const parsed_options& p, variables_map& vm) {
  if (p.description) {
    for (auto& od : p.description->options()) {
      if (vm.find(od->long_name) != vm.end()) continue;
      variable_value vv;
      vv.semantic = od->semantic.get();
      if (od->semantic->apply_default(vv.v)) {
        vv.defaulted = true;
        vm[od->long_name] = vv;
      }
    }
  }
  for (auto& o : p.options) {
    if (o.unregistered) continue;
    const option_description* d = p.description->find(o.string_key, false);
    auto it = vm.find(o.string_key);
    if (it != vm.end() && !it->second.defaulted) continue;  // first store wins
    variable_value vv;
    vv.semantic = d->semantic.get();
    d->semantic->parse(vv.v, o.value);
    vm[o.string_key] = vv;
  }
}

inline void notify(variables_map& vm) {
  for (auto& kv : vm)
    if (kv.second.semantic) kv.second.semantic->notify(kv.second.v);
}

inline parsed_options parse_config_file(std::istream& is, const options_description& desc) {
  parsed_options p;
  p.description = &desc;
  std::string line, section;
  while (std::getline(is, line)) {
    auto h = line.find('#');
    if (h != std::string::npos) line = line.substr(0, h);
    auto trim = [](std::string s) {
      size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
      return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    line = trim(line);
    if (line.empty()) continue;
    if (line[0] == '[') {
      section = trim(line.substr(1, line.find(']') - 1)) + ".";
      continue;
    }
    auto eq = line.find('=');
    if (eq == std::string::npos) throw error("bad config line " + line);
    option o;
    o.string_key = section + trim(line.substr(0, eq));
    o.value.push_back(trim(line.substr(eq + 1)));
    if (!desc.find(o.string_key, false)) throw error("unrecognised option " + o.string_key);
    p.options.push_back(o);
  }
  return p;
}

}  // namespace program_options
}  // namespace boost
