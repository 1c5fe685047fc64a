// yaml.h - stand-in for the part of yaml-cpp that Hamiltonian::IngestBroombridge
// uses (cpp/hamiltonian.cc:8-144): LoadFile, node["key"], node[i], as<T>() and
// iteration over sequences. It reads the YAML subset that Broombridge files use
// (block and flow mappings and sequences, plain and quoted scalars, comments)
// through the project's Broombridge reader, and includes the standard headers
// yaml-cpp brings in (the reference uses std::map and std::set through it).
// TEST INFRASTRUCTURE ONLY: yaml-cpp is a submodule the reference does not vendor.
#ifndef QPE_REF_SHIM_YAML_H_
#define QPE_REF_SHIM_YAML_H_

#include <bitset>
#include <cstdlib>
#include <iostream>
#include <map>
#include <set>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "yaml_subset.h"

namespace YAML {

class Node {
 public:
  Node() : v_(std::make_shared<qpe_yaml::Value>()) {}
  explicit Node(std::shared_ptr<const qpe_yaml::Value> v) : v_(std::move(v)) {}

  Node operator[](const char* key) const {
    if (v_->kind == qpe_yaml::Value::Map)
      for (const auto& kv : v_->map)
        if (kv.first == key) return Node(kv.second);
    return Node();
  }
  Node operator[](const std::string& key) const { return (*this)[key.c_str()]; }
  Node operator[](int i) const {
    if (v_->kind == qpe_yaml::Value::Seq && i >= 0 && (size_t)i < v_->seq.size()) return Node(v_->seq[(size_t)i]);
    return Node();
  }

  template <class T>
  T as() const {
    if (v_->kind != qpe_yaml::Value::Scalar) throw std::runtime_error("YAML shim: not a scalar");
    const std::string& s = v_->scalar;
    if constexpr (std::is_same<T, std::string>::value) {
      return s;
    } else if constexpr (std::is_floating_point<T>::value) {
      return (T)std::strtod(s.c_str(), nullptr);
    } else if constexpr (std::is_unsigned<T>::value) {
      return (T)std::strtoull(s.c_str(), nullptr, 10);
    } else {
      return (T)std::strtoll(s.c_str(), nullptr, 10);
    }
  }

  using const_iterator = std::vector<Node>::const_iterator;
  const_iterator begin() const {
    materialize();
    return items_->begin();
  }
  const_iterator end() const {
    materialize();
    return items_->end();
  }

 private:
  void materialize() const {
    if (items_) return;
    items_ = std::make_shared<std::vector<Node>>();
    if (v_->kind == qpe_yaml::Value::Seq)
      for (const auto& e : v_->seq) items_->push_back(Node(e));
  }
  std::shared_ptr<const qpe_yaml::Value> v_;
  mutable std::shared_ptr<std::vector<Node>> items_;
};

inline Node LoadFile(const std::string& path) { return Node(qpe_yaml::load_file(path)); }

}  // namespace YAML

#endif  // QPE_REF_SHIM_YAML_H_
