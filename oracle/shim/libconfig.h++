// Minimal in-memory stand-in for the libconfig++ Setting/Config classes, just
// enough for the reference's hot-path translation units to compile and run
// inside the oracle harness (test infrastructure; libconfig is not installed
// in this image).  Settings are built programmatically by the harness; there
// is no parser here.
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace libconfig {

class SettingNotFoundException : public std::runtime_error {
 public:
  explicit SettingNotFoundException(const std::string& p) : std::runtime_error("setting not found: " + p) {}
};
class SettingTypeException : public std::runtime_error {
 public:
  explicit SettingTypeException(const std::string& p) : std::runtime_error("setting type: " + p) {}
};

class Setting {
 public:
  enum Type { TypeNone = 0, TypeInt, TypeInt64, TypeFloat, TypeString, TypeBoolean, TypeGroup, TypeArray, TypeList };

  Setting() = default;
  explicit Setting(Type t) : type_(t) {}
  static Setting number(double v) { Setting s(TypeFloat); s.num_ = v; return s; }
  static Setting integer(long v) { Setting s(TypeInt); s.num_ = (double)v; return s; }
  static Setting boolean(bool v) { Setting s(TypeBoolean); s.num_ = v ? 1.0 : 0.0; return s; }
  static Setting string(const std::string& v) { Setting s(TypeString); s.str_ = v; return s; }

  Setting& add(const std::string& name, const Setting& child) {
    auto p = std::make_shared<Setting>(child);
    p->name_ = name;
    children_.push_back(p);
    return *p;
  }
  Setting& add(const Setting& child) { return add("", child); }

  Type getType() const { return type_; }
  bool isGroup() const { return type_ == TypeGroup; }
  bool isArray() const { return type_ == TypeArray; }
  bool isList() const { return type_ == TypeList; }
  bool isAggregate() const { return isGroup() || isArray() || isList(); }
  bool isNumber() const { return type_ == TypeInt || type_ == TypeInt64 || type_ == TypeFloat; }
  bool isScalar() const { return isNumber() || type_ == TypeBoolean || type_ == TypeString; }
  int getLength() const { return (int)children_.size(); }
  const char* getName() const { return name_.c_str(); }
  std::string getPath() const { return name_; }

  bool exists(const std::string& name) const {
    for (auto& c : children_) if (c->name_ == name) return true;
    return false;
  }
  bool exists(const char* name) const { return exists(std::string(name)); }

  Setting& operator[](const std::string& name) const {
    for (auto& c : children_) if (c->name_ == name) return *c;
    throw SettingNotFoundException(name);
  }
  Setting& operator[](const char* name) const { return (*this)[std::string(name)]; }
  Setting& operator[](int i) const {
    if (i < 0 || i >= (int)children_.size()) throw SettingNotFoundException(std::to_string(i));
    return *children_[(size_t)i];
  }
  Setting& lookup(const std::string& name) const { return (*this)[name]; }

  template <typename T>
  bool lookupValue(const std::string& name, T& v) const {
    if (!exists(name)) return false;
    v = (T)(*this)[name];
    return true;
  }
  bool lookupValue(const std::string& name, std::string& v) const {
    if (!exists(name)) return false;
    v = (*this)[name].str_;
    return true;
  }

  const char* c_str() const {
    if (type_ != TypeString) throw SettingTypeException(name_);
    return str_.c_str();
  }
  operator std::string() const { return std::string(c_str()); }
  operator const char*() const { return c_str(); }
  operator double() const { return num(); }
  operator float() const { return (float)num(); }
  operator int() const { return (int)num(); }
  operator long() const { return (long)num(); }
  operator long long() const { return (long long)num(); }
  operator unsigned() const { return (unsigned)num(); }
  operator unsigned long() const { return (unsigned long)num(); }
  operator bool() const { return num() != 0.0; }

 private:
  double num() const {
    if (!(isNumber() || type_ == TypeBoolean)) throw SettingTypeException(name_);
    return num_;
  }
  Type type_ = TypeNone;
  std::string name_;
  double num_ = 0.0;
  std::string str_;
  std::vector<std::shared_ptr<Setting>> children_;
};

class Config {
 public:
  Setting& getRoot() { return root_; }
  const Setting& getRoot() const { return root_; }
  Setting& lookup(const std::string& path) const { return const_cast<Setting&>(root_)[path]; }
  bool exists(const std::string& path) const { return root_.exists(path); }
  void setAutoConvert(bool) {}
  void setOptions(int) {}
  int getOptions() const { return 0; }
  enum { OptionAutoConvert = 1, OptionFsync = 2, OptionSemicolonSeparators = 4, OptionColonAssignmentForGroups = 8,
         OptionColonAssignmentForNonGroups = 16, OptionOpenBraceOnSeparateLine = 32, OptionAllowScientificNotation = 64 };
 private:
  Setting root_{Setting::TypeGroup};
};

}  // namespace libconfig
