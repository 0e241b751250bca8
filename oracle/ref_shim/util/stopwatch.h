// TEST INFRASTRUCTURE: wall-clock stopwatch stand-in.
#pragma once
#include <chrono>
namespace util {
class Stopwatch
{
	using clock = std::chrono::steady_clock;
	clock::time_point t0_;
	double acc_ = 0;
	bool running_ = false;

  public:
	void start()
	{
		t0_ = clock::now();
		running_ = true;
	}
	void stop()
	{
		if (running_)
			acc_ += std::chrono::duration<double>(clock::now() - t0_).count();
		running_ = false;
	}
	double secs() const { return acc_; }
};
struct StopwatchGuard
{
	Stopwatch &sw;
	explicit StopwatchGuard(Stopwatch &s) : sw(s) { sw.start(); }
	~StopwatchGuard() { sw.stop(); }
};
} // namespace util
