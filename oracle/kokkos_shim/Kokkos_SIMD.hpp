// Empty: the reference includes this header but uses none of its contents.
