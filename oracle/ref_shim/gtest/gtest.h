// Minimal stand-in for googletest so that the reference's test translation
// units compile: fixtures derive from testing::Test and every TEST/TEST_F body
// becomes a member function that is compiled but never run.  Assertions
// evaluate nothing.
#pragma once
namespace testing {
class Test {
 public:
  virtual ~Test() {}
 protected:
  virtual void SetUp() {}
  virtual void TearDown() {}
};
}  // namespace testing
#define GSPEC_SHIM_TEST_(fixture, name)                      \
  struct fixture##_##name##_ShimTest : public fixture {      \
    void TestBody();                                         \
  };                                                         \
  void fixture##_##name##_ShimTest::TestBody()
#define TEST_F(fixture, name) GSPEC_SHIM_TEST_(fixture, name)
#define GSPEC_SHIM_SINK(...) do { } while (0)
#define ASSERT_EQ(a, b) GSPEC_SHIM_SINK(a, b)
#define EXPECT_EQ(a, b) GSPEC_SHIM_SINK(a, b)
#define EXPECT_FLOAT_EQ(a, b) GSPEC_SHIM_SINK(a, b)
