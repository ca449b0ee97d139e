// Solver.hpp -- the solver plugin interface and its string-keyed factory.
//
// Same contract as the reference's Solver (src/Base/Solver.hpp:16-31):
// Setup(), Compute(tasks) returning one result per task in task order,
// ApproximateComputationProgress() polled from another thread, and
// nTasksToRequest, the batch size a worker should hand to Compute. Solvers
// register under a name (the reference's SolverFactory::Registrator,
// src/Libraries/TStaticFactory.h:136-144); an unknown name yields nullptr
// (TStaticFactory.h:103-104).
#pragma once

#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace pinco {

class TaskData {
 public:
  virtual ~TaskData() = default;
};

class TaskResults : public TaskData {
 public:
  size_t GetId() const { return id_; }
  void SetId(size_t id) { id_ = id; }

 private:
  size_t id_ = 0;
};

class Solver {
 public:
  virtual ~Solver() = default;
  virtual void Setup() {}
  virtual std::vector<std::unique_ptr<TaskResults>> Compute(const std::vector<std::unique_ptr<TaskData>>& tasks) = 0;
  virtual float ApproximateComputationProgress() const { return 0.0f; }
  size_t nTasksToRequest = 1;
};

template <class Base>
class Factory {
 public:
  using Maker = std::function<Base*()>;

  static std::map<std::string, Maker>& registry() {
    static std::map<std::string, Maker> r;
    return r;
  }
  template <class T>
  static void registerPlugin(const std::string& name) {
    registry()[name] = [] { return static_cast<Base*>(new T()); };
  }
  static Base* makeRawNewInstance(const std::string& name) {
    auto it = registry().find(name);
    return it == registry().end() ? nullptr : it->second();
  }
  static std::unique_ptr<Base> makeUniqueNewInstance(const std::string& name) {
    return std::unique_ptr<Base>(makeRawNewInstance(name));
  }
  static std::vector<std::string> getKeys() {
    std::vector<std::string> k;
    for (auto& e : registry()) k.push_back(e.first);
    return k;
  }
  template <class T>
  struct Registrator {
    explicit Registrator(const std::string& name) { registerPlugin<T>(name); }
  };
};

using SolverFactory = Factory<Solver>;

}  // namespace pinco
