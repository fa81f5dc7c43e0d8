// RenderProgress of the umbreon API: a lock-free progress + cancel channel.
// The inline accessors and the member layout match the reference, so code
// compiled against it reads the same atomics.
#pragma once

#include <atomic>
#include <cstdint>

namespace umbreon {

enum class RenderPhase : int { Idle = 0, Setup, CoarseAo, Primary, GlobalIllum, Edges, Postprocess, Done };

struct RenderPhasePlan {
  float setup = 0.05f;
  float coarseAo = 0.05f;
  float primary = 0.65f;
  float globalIllum = 0.15f;
  float edges = 0.05f;
  float postprocess = 0.05f;
};

class RenderProgress {
 public:
  RenderProgress() = default;
  RenderProgress(const RenderProgress&) = delete;
  RenderProgress& operator=(const RenderProgress&) = delete;

  float fraction() const noexcept;
  RenderPhasePlan phasePlan() const noexcept;
  RenderPhase phase() const noexcept { return static_cast<RenderPhase>(phase_.load(std::memory_order_relaxed)); }
  std::uint64_t unitsDone() const noexcept { return unitsDone_.load(std::memory_order_relaxed); }
  std::uint64_t unitsTotal() const noexcept { return unitsTotal_.load(std::memory_order_relaxed); }
  void requestCancel() noexcept { cancel_.store(true, std::memory_order_relaxed); }
  bool cancelRequested() const noexcept { return cancel_.load(std::memory_order_relaxed); }

  void setPhasePlan(const RenderPhasePlan& plan) noexcept;
  void beginPass(std::uint64_t passIndex, std::uint64_t passCount) noexcept {
    passCount_.store(passCount ? passCount : 1, std::memory_order_relaxed);
    passIndex_.store(passIndex, std::memory_order_relaxed);
    unitsTotal_.store(1, std::memory_order_relaxed);
    unitsDone_.store(0, std::memory_order_relaxed);
    phase_.store(static_cast<int>(RenderPhase::Idle), std::memory_order_relaxed);
  }
  void beginPhase(RenderPhase p, std::uint64_t unitsTotal = 1) noexcept {
    unitsTotal_.store(unitsTotal ? unitsTotal : 1, std::memory_order_relaxed);
    unitsDone_.store(0, std::memory_order_relaxed);
    phase_.store(static_cast<int>(p), std::memory_order_relaxed);
  }
  void advance(std::uint64_t n) noexcept { unitsDone_.fetch_add(n, std::memory_order_relaxed); }
  void advanceTo(std::uint64_t unitsDone) noexcept {
    std::uint64_t cur = unitsDone_.load(std::memory_order_relaxed);
    while (cur < unitsDone &&
           !unitsDone_.compare_exchange_weak(cur, unitsDone, std::memory_order_relaxed, std::memory_order_relaxed)) {
    }
  }
  void markDone() noexcept {
    passIndex_.store(0, std::memory_order_relaxed);
    passCount_.store(1, std::memory_order_relaxed);
    unitsTotal_.store(1, std::memory_order_relaxed);
    unitsDone_.store(1, std::memory_order_relaxed);
    phase_.store(static_cast<int>(RenderPhase::Done), std::memory_order_relaxed);
  }

 private:
  // Phase shares, six 10-bit per-mille slots (setup, coarse AO, primary, GI,
  // edges, post) packed into one word so a plan updates atomically.
  static constexpr int kPlanSlots = 6;
  static constexpr int kPlanBits = 10;
  static constexpr std::uint64_t kPlanMask = (1ull << kPlanBits) - 1;
  static constexpr std::uint64_t kPlanPermille = 1000;
  static constexpr std::uint64_t kDefaultPlanPacked = 50ull | (50ull << kPlanBits) | (650ull << (2 * kPlanBits)) |
                                                      (150ull << (3 * kPlanBits)) | (50ull << (4 * kPlanBits)) |
                                                      (50ull << (5 * kPlanBits));
  std::atomic<int> phase_{static_cast<int>(RenderPhase::Idle)};
  std::atomic<std::uint64_t> unitsDone_{0};
  std::atomic<std::uint64_t> unitsTotal_{1};
  std::atomic<std::uint64_t> passIndex_{0};
  std::atomic<std::uint64_t> passCount_{1};
  std::atomic<std::uint64_t> plan_{kDefaultPlanPacked};
  std::atomic<bool> cancel_{false};
};

const char* toString(RenderPhase p) noexcept;

}  // namespace umbreon
