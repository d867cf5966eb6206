/* Host stand-in for the Sunway athread runtime header, used only to compile
 * the reference's serial drivers on a plain CPU: the two runtime calls the
 * drivers make become no-ops; nothing else in the drivers needs athread. */
#define athread_init() ((void)0)
#define athread_halt() ((void)0)
