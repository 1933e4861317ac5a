// Minimal YAML report writer with the reference's layout
// (ref/src/YAML_Doc.cpp:32-72, YAML_Element.cpp:86-93): "key: value" lines,
// children indented by two spaces per level, a parent's own value empty,
// doubles printed with the stream defaults (6 significant digits), and the
// file named <prefix><YYYY:MM:DD-HH:MM:SS>.yaml in the working directory.
#pragma once

#include <cstdio>
#include <ctime>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace minife_gb300 {

class YamlNode {
 public:
  YamlNode(std::string k, std::string v) : key_(std::move(k)), value_(std::move(v)) {}

  template <typename T>
  YamlNode* add(const std::string& key, const T& value)
  {
    std::ostringstream s;
    s << value;
    return add_str(key, s.str());
  }
  YamlNode* add(const std::string& key, const std::string& value) { return add_str(key, value); }
  YamlNode* add(const std::string& key, const char* value) { return add_str(key, value); }

  YamlNode* get(const std::string& key)
  {
    for (auto& c : children_)
      if (c->key_ == key) return c.get();
    return nullptr;
  }

  std::string print(const std::string& indent) const
  {
    std::string out = indent + key_ + ": " + value_ + "\n";
    for (auto& c : children_) out += c->print(indent + "  ");
    return out;
  }

 protected:
  YamlNode* add_str(const std::string& key, const std::string& value)
  {
    value_.clear();  // a node with children prints an empty value
    children_.emplace_back(new YamlNode(key, value));
    return children_.back().get();
  }
  std::string key_, value_;
  std::vector<std::unique_ptr<YamlNode>> children_;
};

class YamlDoc : public YamlNode {
 public:
  YamlDoc(std::string app, std::string version, std::string file_prefix)
      : YamlNode("", ""), app_(std::move(app)), version_(std::move(version)),
        prefix_(std::move(file_prefix)) {}

  // returns the text and writes the file
  std::string generate()
  {
    std::string y = "Mini-Application Name: " + app_ + "\n";
    y += "Mini-Application Version: " + version_ + "\n";
    for (auto& c : children_) y += c->print("");
    std::time_t raw = std::time(nullptr);
    std::tm* t = std::localtime(&raw);
    char date[32];
    std::snprintf(date, sizeof(date), "%04d:%02d:%02d-%02d:%02d:%02d", t->tm_year + 1900,
                  t->tm_mon + 1, t->tm_mday, t->tm_hour, t->tm_min, t->tm_sec);
    filename_ = "./" + prefix_ + date + ".yaml";
    std::ofstream f(filename_.c_str());
    f << y;
    return y;
  }
  const std::string& filename() const { return filename_; }

 private:
  std::string app_, version_, prefix_, filename_;
};

}  // namespace minife_gb300
