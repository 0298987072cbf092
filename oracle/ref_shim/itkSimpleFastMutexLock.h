// Oracle-only stand-in for ITK's SimpleFastMutexLock (P3MKernel's static caches): a std::mutex.
#pragma once
#include <mutex>
namespace itk {
class SimpleFastMutexLock {
 public:
  void Lock() const { m_Mutex.lock(); }
  void Unlock() const { m_Mutex.unlock(); }

 private:
  mutable std::mutex m_Mutex;
};
}  // namespace itk
